/* C-ABI entry points of libwolkenbase_gb300 and the context they share.
 * Each entry point's counterpart in the reference is named in
 * include/wolkenbase_gb300.h. */
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>
#include "wb_internal.h"
#include "wb_device.cuh"

static thread_local std::string gOpenError;

int wb_fail(wb_ctx *c, int code, const std::string &msg)
{
  if (c)
    c->err = msg;
  else
    gOpenError = msg;
  return code;
}

/* Buffers are stream-ordered allocations on the context's stream: growing
 * one frees the old block after the work queued before it, and neither call
 * waits for other streams (several contexts share a GPU in a server). */
/* Buffers a pass reads or writes in order (sort ping-pong, scratch, the
 * record upload, the tile lists): with paging, a cloud above the budget keeps
 * them in host memory first, so that HBM holds what classify reads at random. */
static bool coldBuffer(const wb_ctx *c, const DevBuf &b)
{
  const DevBuf *cold[] = {&c->rec, &c->key0, &c->key1, &c->idx0, &c->idx1, &c->tmp32, &c->tmp32b,
                          &c->gKey0, &c->gKey1, &c->gVal0, &c->gVal1, &c->tilePts, &c->survivorOf, &c->pointLeaf};
  for (const DevBuf *x : cold)
    if (x == &b)
      return true;
  return false;
}

static const size_t kSpillMin = 1 << 20;   /* smaller scratch buffers stay in HBM while the budget allows */

int wb_ensure(wb_ctx *c, DevBuf &b, size_t bytes)
{
  if (bytes <= b.cap)
    return 0;
  size_t want = bytes + bytes / 8 + 256;
  const size_t devHeld = b.host ? 0 : b.cap, hostHeld = b.host ? b.cap : 0;
  const bool over = c->budget && c->used - devHeld + want > c->budget;
  const bool cold = c->spill_cold && want >= kSpillMin && coldBuffer(c, b);
  if ((over || cold) && c->host_budget && c->host_used - hostHeld + want <= c->host_budget)
  {
    wb_free_buf(c, b);
    cudaError_t e = cudaHostAlloc(&b.p, want, cudaHostAllocMapped | cudaHostAllocPortable);
    if (e == cudaSuccess)
    {
      b.host = true;
      b.cap = want;
      c->host_used += want;
      c->host_peak = std::max(c->host_peak, c->host_used);
      return 0;
    }
    b.p = nullptr;
    cudaGetLastError();
    if (over)
      return wb_fail(c, WB_ENOMEM, std::string("cudaHostAlloc(") + std::to_string(want) + "): " + cudaGetErrorString(e));
  }
  if (over)
    return wb_fail(c, WB_ENOMEM, "device memory budget exceeded (" + std::to_string(c->used - devHeld + want) +
                                     " > " + std::to_string(c->budget) + " bytes)");
  wb_free_buf(c, b);
  cudaError_t e = cudaMallocAsync(&b.p, want, c->stream);
  if (e != cudaSuccess)
  {
    b.p = nullptr;
    cudaGetLastError();
    return wb_fail(c, WB_ENOMEM, std::string("cudaMallocAsync(") + std::to_string(want) + "): " + cudaGetErrorString(e));
  }
  b.cap = want;
  c->used += want;
  return 0;
}

void wb_free_buf(wb_ctx *c, DevBuf &b)
{
  if (!b.p)
    return;
  if (b.host)
  {
    // kernels may still use it: host memory has no stream-ordered free
    cudaStreamSynchronize(c->stream);
    cudaFreeHost(b.p);
    c->host_used -= b.cap;
  }
  else
  {
    cudaFreeAsync(b.p, c->stream);
    c->used -= b.cap;
  }
  b.p = nullptr;
  b.cap = 0;
  b.host = false;
}

void wb_mark(wb_ctx *c, const char *name)
{
  if (!c->profile)
    return;
  cudaEvent_t ev;
  if (cudaEventCreate(&ev) != cudaSuccess)
    return;
  cudaEventRecord(ev, c->stream);
  c->evNames.push_back(name);
  c->events.push_back(ev);
}

void wb_release_buffers(wb_ctx *c)
{
  DevBuf *all[] = {&c->rec, &c->key0, &c->key1, &c->idx0, &c->idx1, &c->tmp32, &c->tmp32b, &c->tmp8, &c->scanTmp,
                   &c->small, &c->lev, &c->cpl, &c->pre, &c->suf, &c->leafId, &c->leafFirst, &c->leafCount,
                   &c->leafLevel, &c->leafKey, &c->leafBox, &c->sidx, &c->sx, &c->sy, &c->sz, &c->xyzd, &c->colOf, &c->gridBounds, &c->pointLeaf,
                   &c->storeOf, &c->survivorOf, &c->nodeChild, &c->nodeBox, &c->nodeStart, &c->nodeIdLevel,
                   &c->tileEx, &c->tileEy, &c->tileLookup, &c->tileStart, &c->tilePts, &c->owner, &c->tileRes,
                   &c->tileHuge, &c->hugePre, &c->scanTot, &c->tileFrm,
                   &c->tileH, &c->tileN, &c->tileNg, &c->label, &c->clsDev, &c->ambiguous, &c->deferred, &c->angleT,
                   &c->flowCache, &c->gKey0, &c->gKey1, &c->gVal0, &c->gVal1, &c->stray, &c->cellStart,
                   &c->gpt, &c->cellRec, &c->superRec, &c->ptSetup, &c->groups, &c->groupCnt, &c->lasAngles,
                   &c->marginBuf, &c->marginRec};
  for (DevBuf *b : all)
    wb_free_buf(c, *b);
  c->used = 0;
}

static void beginRun(wb_ctx *c)
{
  for (cudaEvent_t e : c->events)
    cudaEventDestroy(e);
  c->events.clear();
  c->evNames.clear();
  wb_mark(c, "start");
}

static void endRun(wb_ctx *c)
{
  if (!c->profile || c->events.size() < 2)
    return;
  cudaEventSynchronize(c->events.back());
  c->lastMs.clear();
  c->lastNames.clear();
  for (size_t i = 1; i < c->events.size(); i++)
  {
    float ms = 0;
    cudaEventElapsedTime(&ms, c->events[i - 1], c->events[i]);
    c->lastMs.push_back(ms);
    c->lastNames.push_back(c->evNames[i]);
  }
}

extern "C" {

wb_ctx *wb_open(int device, size_t hbm_budget)
{
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
  {
    cudaGetLastError();
    wb_fail(nullptr, WB_ECUDA, "wb_open: no CUDA device");
    return nullptr;
  }
  if (device < 0 || device >= count)
  {
    wb_fail(nullptr, WB_EINVAL, "wb_open: bad device ordinal");
    return nullptr;
  }
  WbDeviceGuard deviceGuard(device);
  if (!deviceGuard.ok)
  {
    wb_fail(nullptr, WB_ECUDA, "wb_open: cudaSetDevice failed");
    return nullptr;
  }
  wb_ctx *c = new (std::nothrow) wb_ctx;
  if (!c)
    return nullptr;
  c->device = device;
  c->budget = hbm_budget;
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
  {
    wb_fail(nullptr, WB_ECUDA, "wb_open: cudaStreamCreate failed");
    delete c;
    return nullptr;
  }
  c->own_stream = true;
  c->params = wb_params{1.0, 1.0, 0.0, 0.1};
  return c;
}

void wb_close(wb_ctx *c)
{
  if (!c)
    return;
  WbDeviceGuard deviceGuard(c->device);
  if (c->stream)
    cudaStreamSynchronize(c->stream);
  for (cudaEvent_t e : c->events)
    cudaEventDestroy(e);
  wb_release_buffers(c);
  cudaStreamSynchronize(c->stream);
  if (c->hostStage)
    cudaFreeHost(c->hostStage);
  wb_batch_destroy(c->batch);
  if (c->own_stream && c->stream)
    cudaStreamDestroy(c->stream);
  delete c;
}

const char *wb_last_error(const wb_ctx *c)
{
  return c ? c->err.c_str() : gOpenError.c_str();
}

int wb_set_stream(wb_ctx *c, void *s)
{
  if (!c)
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  if (c->stream)
    cudaStreamSynchronize(c->stream);
  if (c->own_stream && c->stream)
    cudaStreamDestroy(c->stream);
  if (s)
  {
    c->stream = (cudaStream_t)s;
    c->own_stream = false;
  }
  else
  {
    cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    c->own_stream = true;
  }
  return 0;
}

int wb_synchronize(wb_ctx *c)
{
  if (!c)
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  return 0;
}

int wb_profile(wb_ctx *c, int enable)
{
  if (!c)
    return WB_EINVAL;
  c->profile = enable != 0;
  return 0;
}

int wb_launch_count(wb_ctx *c, uint64_t *count)
{
  if (!c || !count)
    return WB_EINVAL;
  *count = c->launches;
  return 0;
}

int wb_stage_times(wb_ctx *c, const char **names, float *ms, uint32_t capacity, uint32_t *count)
{
  if (!c)
    return WB_EINVAL;
  uint32_t k = (uint32_t)c->lastMs.size();
  for (uint32_t i = 0; i < k && i < capacity; i++)
  {
    if (names)
      names[i] = c->lastNames[i];
    if (ms)
      ms[i] = c->lastMs[i];
  }
  if (count)
    *count = k;
  return 0;
}

int wb_set_paging(wb_ctx *c, size_t host_budget)
{
  if (!c)
    return WB_EINVAL;
  if (host_budget)
  {
    int mapped = 0, atomics = 0;
    cudaDeviceGetAttribute(&mapped, cudaDevAttrCanMapHostMemory, c->device);
    cudaDeviceGetAttribute(&atomics, cudaDevAttrHostNativeAtomicSupported, c->device);
    if (!mapped || !atomics)
      return wb_fail(c, WB_EINVAL, "wb_set_paging: the device cannot use host memory in place with atomics "
                                   "(needs a coherent CPU link such as NVLink-C2C)");
  }
  c->host_budget = host_budget;
  return 0;
}

int wb_paging_stats(wb_ctx *c, uint64_t *host_bytes, uint64_t *host_peak, uint64_t *device_bytes)
{
  if (!c)
    return WB_EINVAL;
  if (host_bytes)
    *host_bytes = c->host_used;
  if (host_peak)
    *host_peak = c->host_peak;
  if (device_bytes)
    *device_bytes = c->used;
  return 0;
}

int wb_octree_build(wb_ctx *c, const wb_cloud *cloud)
{
  if (!c || !cloud)
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  beginRun(c);
  int rc = wb_build_impl(c, cloud);
  endRun(c);
  return rc;
}

int wb_octree_info(wb_ctx *c, wb_octree_stats *o)
{
  if (!c || !o)
    return WB_EINVAL;
  if (c->stage < 1)
    return wb_fail(c, WB_ESTATE, "wb_octree_info: no octree built");
  memset(o, 0, sizeof *o);
  o->n_points = c->n;
  o->n_distinct = c->nd;
  o->n_leaves = c->n_leaves;
  o->max_depth = c->max_depth;
  for (int k = 0; k < 3; k++)
  {
    o->root_center[k] = c->g.root_c[k];
    o->tile_center[k] = c->g.tile_c[k];
  }
  o->root_side = c->g.root_side;
  o->tile_side = c->g.tile_side;
  wb_params p = c->params;
  int idx, lo, hi;
  double sp;
  wb_snake_size(c->g.tile_side, p.tile_size > 0 ? p.tile_size : 1.0, &idx, &sp, &lo, &hi);
  o->spacing = sp;
  o->n_tiles = (uint64_t)((int64_t)hi - lo + 1);
  o->tile_lo = lo;
  o->tile_hi = hi;
  return 0;
}

int wb_octree_leaves(wb_ctx *c, double *cs, uint32_t *first, uint32_t *count)
{
  if (!c)
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  if (c->stage < 1)
    return wb_fail(c, WB_ESTATE, "wb_octree_leaves: no octree built");
  uint64_t L = c->n_leaves;
  if (L == 0)
    return 0;
  std::vector<uint64_t> key(L);
  std::vector<uint8_t> lev(L);
  WB_CUDA(c, cudaMemcpyAsync(key.data(), c->leafKey.p, L * 8, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaMemcpyAsync(lev.data(), c->leafLevel.p, L, cudaMemcpyDefault, c->stream));
  if (first)
    WB_CUDA(c, cudaMemcpyAsync(first, c->leafFirst.p, L * 4, cudaMemcpyDefault, c->stream));
  if (count)
    WB_CUDA(c, cudaMemcpyAsync(count, c->leafCount.p, L * 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (cs)
    for (uint64_t l = 0; l < L; l++)
    {
      // Octree::cube: centre = parent centre +- side/4 per level, computed exactly
      int lv = lev[l];
      uint32_t ix = 0, iy = 0, iz = 0;
      for (int d = 1; d <= lv; d++)
      {
        int oct = (int)((key[l] >> (63 - 3 * d)) & 7);
        ix = (ix << 1) | (oct & 1);
        iy = (iy << 1) | ((oct >> 1) & 1);
        iz = (iz << 1) | ((oct >> 2) & 1);
      }
      double side = ldexp(c->g.root_side, -lv);
      cs[4 * l + 0] = c->g.root_lo[0] + ((double)ix + 0.5) * side;
      cs[4 * l + 1] = c->g.root_lo[1] + ((double)iy + 0.5) * side;
      cs[4 * l + 2] = c->g.root_lo[2] + ((double)iz + 0.5) * side;
      cs[4 * l + 3] = side;
    }
  return 0;
}

int wb_octree_point_leaf(wb_ctx *c, uint32_t *out)
{
  if (!c || (!out && c->n))
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  if (c->stage < 1)
    return wb_fail(c, WB_ESTATE, "wb_octree_point_leaf: no octree built");
  if (c->n)
  {
    int rc = wb_point_leaf_map(c);
    if (rc)
      return rc;
    WB_CUDA(c, cudaMemcpyAsync(out, c->pointLeaf.p, c->n * 4, cudaMemcpyDefault, c->stream));
    WB_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return 0;
}

int wb_octree_store_order(wb_ctx *c, uint32_t *out)
{
  if (!c || (!out && c->nd))
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  if (c->stage < 1)
    return wb_fail(c, WB_ESTATE, "wb_octree_store_order: no octree built");
  if (c->nd)
  {
    WB_CUDA(c, cudaMemcpyAsync(out, c->sidx.p, c->nd * 4, cudaMemcpyDefault, c->stream));
    WB_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return 0;
}

int wb_octree_find_block(wb_ctx *c, const double *xyz, uint64_t m, int64_t *leaf)
{
  if (!c || (m && (!xyz || !leaf)))
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  if (c->stage < 1)
    return wb_fail(c, WB_ESTATE, "wb_octree_find_block: no octree built");
  return wb_find_block_impl(c, xyz, m, leaf);
}

int wb_scan_tiles(wb_ctx *c, const wb_params *p)
{
  if (!c || !p)
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  beginRun(c);
  int rc = wb_scan_impl(c, p);
  endRun(c);
  return rc;
}

int wb_tiles(wb_ctx *c, wb_tile *out, uint64_t capacity, uint64_t *count)
{
  if (!c)
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  if (c->stage < 2)
    return wb_fail(c, WB_ESTATE, "wb_tiles: scan the tiles first");
  uint64_t T = c->n_tiles;
  if (count)
    *count = T;
  if (!out)
    return 0;
  if (capacity < T)
    return wb_fail(c, WB_EINVAL, "wb_tiles: capacity below the tile count");
  std::vector<TileRes> r(T);
  WB_CUDA(c, cudaMemcpyAsync(r.data(), c->tileRes.p, T * sizeof(TileRes), cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  for (uint64_t k = 0; k < T; k++)
  {
    wb_tile &t = out[k];
    t.ex = c->flowHostEx[k];
    t.ey = c->flowHostEy[k];
    t.n_points = r[k].nPoints;
    t.n_ground = r[k].nGround;
    t.tree_flags = r[k].treeFlags;
    t.pad = 0;
    t.density = r[k].density;
    t.h_scan = r[k].hScan;
    t.hyperboloid_size = r[k].h;
    t.height = r[k].height;
  }
  return 0;
}

int wb_classify(wb_ctx *c, const wb_params *p, uint8_t *cls, int onDevice)
{
  if (!c || !p)
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  beginRun(c);
  int rc = wb_classify_impl(c, p, cls, onDevice);
  if (rc == 0 && !onDevice)
  {
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
      rc = wb_fail(c, WB_ECUDA, std::string("wb_classify: ") + cudaGetErrorString(e));
  }
  endRun(c);
  return rc;
}

int wb_classify_ex(wb_ctx *c, const wb_params *p, uint8_t *cls, int onDevice, float *margin)
{
  if (!c || !p)
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  if (margin && onDevice && c->n && !wb_device_accessible(margin))
    return wb_fail(c, WB_EINVAL, "wb_classify_ex: device margins must be device memory");
  c->marginDst = margin;
  beginRun(c);
  int rc = wb_classify_impl(c, p, cls, onDevice);
  if (rc == 0 && !onDevice)
  {
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
      rc = wb_fail(c, WB_ECUDA, std::string("wb_classify_ex: ") + cudaGetErrorString(e));
  }
  endRun(c);
  c->marginDst = nullptr;
  return rc;
}

int wb_set_tuning(wb_ctx *c, const wb_tuning *t)
{
  if (!c || !t)
    return WB_EINVAL;
  if (t->shape >= WB_N_SHAPES || t->shape < -1 || t->chunk < 0 || t->grid_points < 0)
    return wb_fail(c, WB_EINVAL, "wb_set_tuning: shape in 0..WB_N_SHAPES-1 (or -1), chunk and grid_points >= 0");
  if (t->shape >= 0)
    c->shape = t->shape;
  if (t->chunk > 0)
    c->chunk = t->chunk;
  if (t->grid_points > 0)
    c->grid_points = t->grid_points;
  return 0;
}

int wb_set_precision(wb_ctx *c, int mode)
{
  if (!c)
    return WB_EINVAL;
  if (mode != WB_PRECISION_EXACT && mode != WB_PRECISION_FP32)
    return wb_fail(c, WB_EINVAL, "wb_set_precision: WB_PRECISION_EXACT or WB_PRECISION_FP32");
  c->precision = mode;
  return 0;
}

int wb_tile_planes(wb_ctx *c, double *abc, uint64_t capacity)
{
  if (!c || !abc)
    return WB_EINVAL;
  if (c->stage < 2)
    return wb_fail(c, WB_ESTATE, "wb_tile_planes: scan the tiles first");
  uint64_t T = c->n_tiles;
  if (capacity < T)
    return wb_fail(c, WB_EINVAL, "wb_tile_planes: capacity below the tile count");
  WbDeviceGuard deviceGuard(c->device);
  std::vector<TileRes> r(T);
  if (T)
    WB_CUDA(c, cudaMemcpyAsync(r.data(), c->tileRes.p, T * sizeof(TileRes), cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  for (uint64_t k = 0; k < T; k++)
    for (int i = 0; i < 3; i++)
      abc[3 * k + i] = r[k].plane[i];
  return 0;
}

int wb_get_tuning(wb_ctx *c, wb_tuning *t)
{
  if (!c || !t)
    return WB_EINVAL;
  t->shape = c->shape;
  t->chunk = c->chunk;
  t->grid_points = c->grid_points;
  return 0;
}

int wb_autotune(wb_ctx *c, const wb_params *p)
{
  if (!c || !p)
    return WB_EINVAL;
  if (c->stage < 2)
    return wb_fail(c, WB_ESTATE, "wb_autotune: scan the tiles first");
  WbDeviceGuard deviceGuard(c->device);
  std::string err;
  int rc = 0;
  if (!c->batch && (rc = wb_batch_create(c->device, &c->batch, err)))
    return wb_fail(c, rc, err);
  // stage against the context's own device class buffer; the timing runs
  // write labels only, never class bytes
  if ((rc = wb_ensure(c, c->clsDev, c->n + 64)))
    return rc;
  int shape = c->shape, chunk = c->chunk;
  double gp = c->grid_points;
  WbTuneJob job{c, p, (uint8_t *)c->clsDev.p, 1};
  if ((rc = wb_classify_stage(c, p, (uint8_t *)c->clsDev.p, 1)) ||
      (rc = wb_autotune_jobs(c->batch, &job, 1, c->stream, &shape, &chunk, &gp, err)))
    return wb_fail(c, rc, "wb_autotune: " + (err.empty() ? c->err : err));
  c->shape = shape;
  c->chunk = chunk;
  c->grid_points = gp;
  c->clsStaged = false;
  return 0;
}

int wb_classify_cloud(wb_ctx *c, const wb_cloud *cloud, const wb_params *p, uint8_t *cls)
{
  if (!c || !cloud || !p)
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  beginRun(c);
  int rc = wb_build_impl(c, cloud);
  if (rc == 0)
    rc = wb_scan_impl(c, p);
  if (rc == 0)
    rc = wb_classify_impl(c, p, cls, cloud->device_resident ? 1 : 0);
  if (rc == 0)
  {
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
      rc = wb_fail(c, WB_ECUDA, std::string("wb_classify_cloud: ") + cudaGetErrorString(e));
  }
  endRun(c);
  return rc;
}

}  // extern "C"

/* ---- Octree::findBlock for arbitrary positions ---- */
namespace
{
__global__ void findBlockKernel(const double *__restrict__ xyz, uint64_t m, WbRoot r, const uint64_t *__restrict__ leafKey,
                                const uint8_t *__restrict__ leafLev, uint64_t L, int64_t *__restrict__ out)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t ix = wb_cell_index(xyz[3 * i], r.lo[0], r.cell);
    uint32_t iy = wb_cell_index(xyz[3 * i + 1], r.lo[1], r.cell);
    uint32_t iz = wb_cell_index(xyz[3 * i + 2], r.lo[2], r.cell);
    uint64_t key = wb_morton(ix, iy, iz);
    // last leaf whose key prefix is <= key
    uint64_t lo = 0, hi = L;
    while (lo < hi)
    {
      uint64_t mid = (lo + hi) / 2;
      if (leafKey[mid] <= key)
        lo = mid + 1;
      else
        hi = mid;
    }
    int64_t res = -1;
    if (lo > 0)
    {
      uint64_t l = lo - 1;
      int lv = leafLev[l];
      if ((key >> (63 - 3 * lv)) == (leafKey[l] >> (63 - 3 * lv)))
        res = (int64_t)l;
    }
    out[i] = res;
  }
}
}  // namespace

/* ---- findBlock with static staging: no allocation on the call path ----
 * The staging lives in file-scope device arrays.  Host code must not pass the
 * array names to a kernel (on the host they are only stand-ins); the device
 * addresses are looked up once per device with cudaGetSymbolAddress. */
static __device__ __align__(256) double gFindStaticIn[3 * WB_FIND_BLOCK_STATIC_MAX];
static __device__ __align__(256) int64_t gFindStaticOut[WB_FIND_BLOCK_STATIC_MAX];

namespace
{
struct StaticSlots
{
  double *in = nullptr;
  int64_t *out = nullptr;
};
std::mutex gStaticMutex;
StaticSlots gStaticByDevice[64];
}  // namespace

static int staticSlots(wb_ctx *c, StaticSlots &s)
{
  if (c->device < 0 || c->device >= 64)
    return wb_fail(c, WB_EINVAL, "wb_octree_find_block_static: device ordinal above 63");
  std::lock_guard<std::mutex> lock(gStaticMutex);
  StaticSlots &d = gStaticByDevice[c->device];
  if (!d.in)
  {
    void *pin = nullptr, *pout = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&pin, gFindStaticIn);
    if (e != cudaSuccess)
      return wb_fail(c, WB_ECUDA, std::string("cudaGetSymbolAddress(staging in): ") + cudaGetErrorString(e));
    e = cudaGetSymbolAddress(&pout, gFindStaticOut);
    if (e != cudaSuccess)
      return wb_fail(c, WB_ECUDA, std::string("cudaGetSymbolAddress(staging out): ") + cudaGetErrorString(e));
    d.in = (double *)pin;
    d.out = (int64_t *)pout;
  }
  s = d;
  return 0;
}

extern "C" int wb_octree_find_block_static(wb_ctx *c, const double *xyz, uint64_t m, int64_t *leaf)
{
  if (!c || (m && (!xyz || !leaf)))
    return WB_EINVAL;
  if (c->stage < 1)
    return wb_fail(c, WB_ESTATE, "wb_octree_find_block_static: no octree built");
  if (m > WB_FIND_BLOCK_STATIC_MAX)
    return wb_fail(c, WB_EINVAL, "wb_octree_find_block_static: " + std::to_string(m) + " positions exceed the " +
                                     std::to_string(WB_FIND_BLOCK_STATIC_MAX) + "-entry static staging array");
  if (m == 0)
    return 0;
  WbDeviceGuard deviceGuard(c->device);
  StaticSlots s;
  int rc = staticSlots(c, s);
  if (rc)
    return rc;
  WbRoot r;
  for (int k = 0; k < 3; k++)
    r.lo[k] = c->g.root_lo[k];
  r.side = c->g.root_side;
  r.cell = c->g.cell;
  WB_CUDA(c, cudaMemcpyAsync(s.in, xyz, m * 24, cudaMemcpyDefault, c->stream));
  { findBlockKernel<<<(unsigned)std::min<uint64_t>((m + 255) / 256, 4096), 256, 0, c->stream>>>(
        s.in, m, r, (const uint64_t *)c->leafKey.p, (const uint8_t *)c->leafLevel.p, c->n_leaves, s.out); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  WB_CUDA(c, cudaMemcpyAsync(leaf, s.out, m * 8, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  return 0;
}

int wb_find_block_impl(wb_ctx *c, const double *xyz, uint64_t m, int64_t *leaf)
{
  if (m == 0)
    return 0;
  int rc;
  DevBuf in, out;
  if ((rc = wb_ensure(c, in, m * 24)) || (rc = wb_ensure(c, out, m * 8)))
  {
    wb_free_buf(c, in);
    return rc;
  }
  WbRoot r;
  for (int k = 0; k < 3; k++)
    r.lo[k] = c->g.root_lo[k];
  r.side = c->g.root_side;
  r.cell = c->g.cell;
  cudaMemcpyAsync(in.p, xyz, m * 24, cudaMemcpyDefault, c->stream);
  { findBlockKernel<<<(unsigned)std::min<uint64_t>((m + 255) / 256, 4096), 256, 0, c->stream>>>(
      (const double *)in.p, m, r, (const uint64_t *)c->leafKey.p, (const uint8_t *)c->leafLevel.p, c->n_leaves,
      (int64_t *)out.p); ++c->launches; }
  cudaMemcpyAsync(leaf, out.p, m * 8, cudaMemcpyDefault, c->stream);
  wb_free_buf(c, in);
  wb_free_buf(c, out);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess)
    return wb_fail(c, WB_ECUDA, std::string("wb_octree_find_block: ") + cudaGetErrorString(e));
  return 0;
}

/* ---- device arithmetic self-checks ---- */
#include "angle_tables.h"
namespace
{
__global__ void atanCheckKernel(const double *yx, uint64_t m, const double *tab, int32_t *out)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = wb_atan2i(yx[2 * i], yx[2 * i + 1], tab, tab + 511, tab + 1023, WB_ATAN_SCALE_HI, WB_ATAN_SCALE_LO);
}
__global__ void dirCheckKernel(const int32_t *d, float sx, float sy, uint64_t m, uint32_t *out)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
  {
    float dx = (float)d[2 * i] * sx, dy = (float)d[2 * i + 1] * sy;
    out[i] = (uint32_t)__float2int_rn(wb_dir_units_f32(dy, dx)) & 0x7fffffffu;
  }
}
__global__ void hypotCheckKernel(const double *ab, uint64_t m, double *out)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = wb_hypot(ab[2 * i], ab[2 * i + 1]);
}
__global__ void hypCheckKernel(double vx, double vy, double vz, double r, double s, const double *xyz, uint64_t m,
                               uint8_t *out)
{
  double por = r * (s * s);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
    out[i] = wb_hyp_in(vx + 0, vy + 0, vz + por, por * por, s, xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
}

template <class F>
int withDevice(size_t inBytes, const void *in, size_t outBytes, void *out, F launch)
{
  void *din = nullptr, *dout = nullptr;
  if (cudaMalloc(&din, inBytes + 16) != cudaSuccess)
    return WB_ENOMEM;
  if (cudaMalloc(&dout, outBytes + 16) != cudaSuccess)
  {
    cudaFree(din);
    return WB_ENOMEM;
  }
  int rc = 0;
  if (cudaMemcpy(din, in, inBytes, cudaMemcpyDefault) != cudaSuccess)
    rc = WB_ECUDA;
  if (!rc)
  {
    launch(din, dout);
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, dout, outBytes, cudaMemcpyDefault) != cudaSuccess)
      rc = WB_ECUDA;
  }
  cudaFree(din);
  cudaFree(dout);
  return rc;
}
}  // namespace

extern "C" {
int wb_check_atan2i(const double *yx, uint64_t m, int32_t *out)
{
  if (!m)
    return 0;
  if (!yx || !out)
    return WB_EINVAL;
  double *tab = nullptr;
  if (cudaMalloc(&tab, 1535 * 8) != cudaSuccess)
    return WB_ENOMEM;
  cudaMemcpy(tab, kWbTan, 511 * 8, cudaMemcpyDefault);
  cudaMemcpy(tab + 511, kWbSin, 512 * 8, cudaMemcpyDefault);
  cudaMemcpy(tab + 1023, kWbCos, 512 * 8, cudaMemcpyDefault);
  int rc = withDevice(m * 16, yx, m * 4, out, [&](void *din, void *dout) {
    atanCheckKernel<<<(unsigned)((m + 255) / 256 < 4096 ? (m + 255) / 256 : 4096), 256>>>((const double *)din, m, tab,
                                                                                         (int32_t *)dout);
  });
  cudaFree(tab);
  return rc;
}

int wb_check_dir_f32(const int32_t *dxy, double sx, double sy, uint64_t m, uint32_t *out)
{
  if (!m)
    return 0;
  if (!dxy || !out)
    return WB_EINVAL;
  return withDevice(m * 8, dxy, m * 4, out, [&](void *din, void *dout) {
    dirCheckKernel<<<(unsigned)((m + 255) / 256 < 4096 ? (m + 255) / 256 : 4096), 256>>>(
        (const int32_t *)din, (float)sx, (float)sy, m, (uint32_t *)dout);
  });
}

int wb_check_hypot(const double *ab, uint64_t m, double *out)
{
  if (!m)
    return 0;
  if (!ab || !out)
    return WB_EINVAL;
  return withDevice(m * 16, ab, m * 8, out, [&](void *din, void *dout) {
    hypotCheckKernel<<<(unsigned)((m + 255) / 256 < 4096 ? (m + 255) / 256 : 4096), 256>>>((const double *)din, m,
                                                                                          (double *)dout);
  });
}

int wb_check_hyperboloid(const double *v, double r, double s, const double *xyz, uint64_t m, uint8_t *out)
{
  if (!m)
    return 0;
  if (!v || !xyz || !out)
    return WB_EINVAL;
  return withDevice(m * 24, xyz, m, out, [&](void *din, void *dout) {
    hypCheckKernel<<<(unsigned)((m + 255) / 256 < 4096 ? (m + 255) / 256 : 4096), 256>>>(
        v[0], v[1], v[2], r, s, (const double *)din, m, (uint8_t *)dout);
  });
}
}  // extern "C"

/* Internal declarations of libwolkenbase_gb300: the context, device buffers,
 * host-side geometry set-up and the kernel launchers of each stage. */
#ifndef WB_INTERNAL_H
#define WB_INTERNAL_H
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <string>
#include <vector>
#include "wolkenbase_gb300.h"

/* Grow-only device buffer; capacity is charged against the context budget. */
struct DevBuf
{
  void *p = nullptr;
  size_t cap = 0;
  bool host = false;   /* pinned host memory the kernels use in place (paging) */
};

struct WbGeom
{
  double off[3], scale[3], unit;
  double root_c[3], root_side;
  double root_lo[3], cell;          /* root lo corner and level-21 cell edge */
  double tile_c[3], tile_side;      /* cube given to Flowsnake::setSize      */
  double spacing;
  int snake_idx, tile_lo, tile_hi;
  bool exact_ints;                  /* decode is strictly increasing in X, Y, Z */
};

/* Column grid over the point store (wb_grid.cu). */
struct GridInfo
{
  double x0 = 0, y0 = 0, cell = 1;
  int nx = 0, ny = 0;
  uint64_t ncell = 0, nStray = 0;
  int zminInt = 0;
  int32_t imin[3] = {0, 0, 0}, imax[3] = {0, 0, 0};   /* record-integer extent of the cloud */
  /* super-cells: blocks of WB_SUPER x WB_SUPER columns with their own bounds */
  int snx = 0, sny = 0;
  uint64_t nGroups = 0;             /* column groups of up to 32 points */
};
#define WB_SUPER 3
/* a warp tests a super-cell's columns with one lane each */
static_assert(WB_SUPER * WB_SUPER <= 32, "WB_SUPER^2 columns must fit the lanes of a warp");

struct wb_ctx
{
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  size_t budget = 0;
  std::atomic<size_t> used{0};      /* device bytes held (read by a server's scheduler) */
  /* paging (wb_set_paging): buffers beyond the HBM budget in pinned host memory */
  size_t host_budget = 0;
  size_t host_used = 0, host_peak = 0;
  bool spill_cold = false;          /* this cloud needs more than the budget: scratch buffers go to the host */
  std::string err;
  int sm_count = 0;
  uint64_t launches = 0;            /* kernels launched by this context */

  /* state */
  int stage = 0;                    /* 0 empty, 1 built, 2 scanned, 3 classified */
  uint64_t n = 0, nd = 0, n_leaves = 0, n_nodes = 0, n_tiles = 0;
  uint32_t max_depth = 0;
  uint64_t n_ambiguous = 0;         /* points the exact classify pass re-ran */
  WbGeom g{};
  wb_params params{};
  int precision = WB_PRECISION_EXACT;   /* wb_set_precision */

  /* named device buffers */
  DevBuf rec, key0, key1, idx0, idx1, tmp32, tmp32b, tmp8, scanTmp, small;
  DevBuf lev, cpl, pre, suf, leafId;
  DevBuf leafFirst, leafCount, leafLevel, leafKey, leafBox;
  DevBuf sidx, sx, sy, sz, pointLeaf, storeOf, survivorOf;
  /* decoded coordinates of the stored points, three planes of nd doubles
     (x, y, z), each the reference's (offset + scale * X) * unit */
  DevBuf xyzd;
  DevBuf colOf;   /* column {i, j} of each stored point (unclamped, within +-1e9) */
  DevBuf gridBounds;   /* record-integer column boundaries and root-cube faces */
  DevBuf nodeChild, nodeBox, nodeStart, nodeIdLevel;
  DevBuf tileEx, tileEy, tileLookup, tileStart, tilePts, owner, tileRes, tileH, tileN, tileNg, tileHuge, hugePre,
      scanTot, tileFrm;
  DevBuf label, clsDev, ambiguous, deferred, angleT;
  /* column grid (wb_grid.cu): gpt holds one int4 {X, Y, Z, store position |
     stray bit} per point in column order; cellRec two int4 per column,
     {x0, y0, x1, y1} and {zmin, begin, end, flags}, x0 == INT32_MAX for an
     empty column; superRec the same two int4 per super-cell */
  DevBuf gKey0, gKey1, gVal0, gVal1, stray, cellStart, gpt, cellRec, superRec, ptSetup;
  DevBuf groups, groupCnt;          /* column groups: uint2 {column, first point} of up to 32 points */
  GridInfo grid;
  /* fused fast-pass settings (wb_set_tuning; a server's autotuner picks them
     per batch): kernel shape, work chunk and points per grid column */
  int shape = 0, chunk = 1;
  double grid_points = 64;
  struct WbBatch *batch = nullptr;  /* job table of the batch-of-one launch */
  double grid_bounds[4] = {0, 0, 0, 0};   /* x0, y0, x1, y1 the column grid spans */
  DevBuf flowCache;
  DevBuf lasAngles;                 /* scan-angle tables of the LAS decode and writer */
  void *hostStage = nullptr;        /* pinned staging for per-block tables (grow-only) */
  size_t hostStageCap = 0;
  std::vector<int32_t> flowHostEx, flowHostEy;   /* cached flowsnake order for snake_idx */
  int flowIdxCached = -1;
  int lookupX0 = 0, lookupY0 = 0, lookupW = 0, lookupH = 0;

  /* classify arguments formed by wb_classify_stage for a fused launch */
  alignas(16) unsigned char clsArgs[768];
  bool clsStaged = false;
  uint8_t *clsHost = nullptr;       /* host destination of the class bytes, or NULL */
  const uint8_t *clsFinal = nullptr; /* device class bytes of the last classify (per record) */
  uint64_t n_ground = 0;
  /* wb_classify_ex: where the decision margins go (NULL: not formed) */
  float *marginDst = nullptr;
  DevBuf marginBuf, marginRec;

  /* profiling */
  bool profile = false;
  std::vector<const char *> evNames;
  std::vector<cudaEvent_t> events;
  std::vector<float> lastMs;
  std::vector<const char *> lastNames;
};

/* Per-tile results of scan/postscan/classify (Tile, tile.h:27-35). */
struct TileRes
{
  int32_t nPoints, nGround, treeFlags, pad;
  double density, hScan, h, height;
  double plane[3];   /* least-squares plane z = a*x + b*y + c, x and y from the tile centre */
};

/* Makes `device` current for the guard's lifetime and gives the caller's
 * current device back when it ends, so that no entry point leaves the host
 * application on another device than the one it was using. */
struct WbDeviceGuard
{
  int prev = -1;
  bool ok = true;
  explicit WbDeviceGuard(int device)
  {
    if (cudaGetDevice(&prev) != cudaSuccess)
    {
      prev = -1;
      cudaGetLastError();
    }
    if (prev != device)
      ok = cudaSetDevice(device) == cudaSuccess;
  }
  WbDeviceGuard(const WbDeviceGuard &) = delete;
  WbDeviceGuard &operator=(const WbDeviceGuard &) = delete;
  ~WbDeviceGuard()
  {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev)
      cudaSetDevice(prev);
  }
};

/* error helpers */
int wb_fail(wb_ctx *c, int code, const std::string &msg);
#define WB_CUDA(c, call)                                                        \
  do                                                                            \
  {                                                                             \
    cudaError_t e__ = (call);                                                   \
    if (e__ != cudaSuccess)                                                     \
      return wb_fail((c), WB_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
  } while (0)

int wb_ensure(wb_ctx *c, DevBuf &b, size_t bytes);
void wb_free_buf(wb_ctx *c, DevBuf &b);   /* stream-ordered free (host buffers after a sync) */

/* A scratch buffer of one call, freed when it leaves scope. */
struct WbScratch
{
  wb_ctx *c;
  DevBuf b;
  explicit WbScratch(wb_ctx *ctx) : c(ctx) {}
  WbScratch(const WbScratch &) = delete;
  WbScratch &operator=(const WbScratch &) = delete;
  ~WbScratch() { wb_free_buf(c, b); }
};
void wb_release_buffers(wb_ctx *c);       /* frees every buffer of c */
void wb_mark(wb_ctx *c, const char *name);   /* profiling event after a stage */

/* host geometry (wb_geom.cpp) */
void wb_size_fit(const double mn[3], const double mx[3], double center[3], double *side);
void wb_tile_cube(const double mn[3], const double mx[3], double center[3], double *side);
void wb_snake_size(const double tile_side, double desired, int *idx, double *spacing, int *lo, int *hi);
void wb_flowsnake_order(int idx, std::vector<int32_t> &ex, std::vector<int32_t> &ey);

/* primitives (wb_prims.cu) */
int wb_exclusive_scan_u32(wb_ctx *c, const uint32_t *in, uint32_t *out, uint64_t n, uint32_t *total_dev);
int wb_copy_in(wb_ctx *c, void *dst, const void *src, size_t bytes);   /* caller's host buffer -> device */
bool wb_device_accessible(const void *p);   /* device, managed or device-mapped host memory */
int wb_radix_sort_pairs(wb_ctx *c, uint64_t *&keys, uint32_t *&vals, uint64_t *keysAlt, uint32_t *valsAlt,
                        uint64_t n, int beginBit, int endBit);

/* stages */
int wb_point_leaf_map(wb_ctx *c);   /* point -> leaf map into c->pointLeaf */
int wb_build_impl(wb_ctx *c, const wb_cloud *cloud);
int wb_grid_impl(wb_ctx *c, double x0, double y0, double x1, double y1);
int wb_scan_impl(wb_ctx *c, const wb_params *p);
int wb_classify_impl(wb_ctx *c, const wb_params *p, uint8_t *cls, int onDevice);
int wb_find_block_impl(wb_ctx *c, const double *xyz, uint64_t m, int64_t *leaf);

/* fused classify of many jobs in one captured graph (wb_classify.cu) */
#define WB_BATCH_MAX 512
struct WbBatch;
int wb_batch_create(int device, WbBatch **out, std::string &err);
void wb_batch_destroy(WbBatch *b);
int wb_classify_stage(wb_ctx *c, const wb_params *p, uint8_t *cls, int onDevice);
int wb_batch_launch(WbBatch *b, wb_ctx *const *jobs, int k, cudaStream_t s, int shape, int chunk,
                    uint64_t *launches, std::string &err);
void wb_batch_collect(WbBatch *b, wb_ctx *const *jobs, int k);
/* Kernel shapes of the fused fast pass: warps per block and a register cap
 * (minimum resident blocks per SM, 0 = none). */
struct WbShape
{
  int warps, minBlocks;
};
extern const WbShape kWbShapes[WB_N_SHAPES];
/* Times the fused fast pass alone over the first `sample` points of the
 * staged jobs (set-up included, untimed); the jobs' ambiguous lists are
 * cleared afterwards, so the batch can be launched normally. */
int wb_batch_time(WbBatch *b, wb_ctx *const *jobs, int k, uint64_t sample, int shape, int chunk, cudaStream_t s,
                  float *ms, std::string &err);
struct WbTuneJob
{
  wb_ctx *c;
  const wb_params *p;
  uint8_t *cls;
  int onDevice;
};
int wb_autotune_jobs(WbBatch *b, const WbTuneJob *jobs, int k, cudaStream_t s, int *shape, int *chunk,
                     double *gridPoints, std::string &err);

#endif

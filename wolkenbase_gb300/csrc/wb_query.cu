/* Shape queries over the device-resident octree: Octree::findBlocks
 * (octree.cpp:234-251) and OctStore::pointsIn (octree.cpp:1214-1242) for the
 * two shapes the classification path asks about, a Cylinder (shape.cpp:
 * 214-238) and a downward Hyperboloid (shape.cpp:119-159).
 *
 * findBlocks descends from the root into every octant whose cube the shape
 * intersects (Shape::intersect: the shape holds the cube's closest point,
 * shape.cpp:63-66).  For these convex shapes a cube that meets the shape has
 * every ancestor meeting it too, so the blocks found are exactly the leaves
 * whose own cube meets the shape, in depth-first order -- the leaf table's
 * order.  pointsIn then takes a whole block when all eight corners of its
 * cube are inside (Shape::in(Cube), shape.cpp:50-61) and otherwise every
 * point the shape holds, in store order; sorted=true orders the result by
 * height (the reference's std::sort by z leaves ties in no particular order;
 * here ties keep the unsorted order).
 *
 * One warp per leaf: the cube tests on lane 0's doubles, the per-point tests
 * across the lanes with ballot compaction (store order kept), a scan of the
 * per-leaf counts, a second pass writing the record indices.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include "wb_internal.h"
#include "wb_device.cuh"

namespace
{
struct QShape
{
  int kind;
  double cx, cy, cz;   /* cylinder: centre (z unused); hyperboloid: centre v + (0, 0, por) */
  double r;            /* cylinder radius */
  double por2, slope;  /* hyperboloid */
};

struct QArgs
{
  QShape s;
  uint64_t L;
  const uint64_t *leafKey;
  const uint8_t *leafLev;
  const uint32_t *first, *count;
  const int32_t *sx, *sy, *sz;
  const uint32_t *sidx;
  double rootLo[3], rootSide;
  double off[3], scale[3], unit;
};

__device__ __forceinline__ bool shapeIn(const QShape &s, double x, double y, double z)
{
  if (s.kind == WB_SHAPE_CYLINDER)
    return wb_hypot(s.cx - x, s.cy - y) <= s.r;
  return wb_hyp_in(s.cx, s.cy, s.cz, s.por2, s.slope, x, y, z);
}

/* Shape::intersect (shape.cpp:63-66) with closestPoint of the Cylinder
 * (shape.cpp:220-238: the cube's centre height) or the Hyperboloid
 * (shape.cpp:137-159: the cube's bottom for a downward one, top otherwise). */
__device__ __forceinline__ bool shapeMeets(const QShape &s, double cx, double cy, double cz, double side)
{
  const double x = wb_clamp_toward(s.cx, cx, side), y = wb_clamp_toward(s.cy, cy, side);
  double z = cz;
  if (s.kind == WB_SHAPE_HYPERBOLOID)
  {
    if (s.slope > 0)
      z -= side / 2;
    if (s.slope < 0)
      z += side / 2;
  }
  return shapeIn(s, x, y, z);
}

/* Shape::in(Cube): all eight corners inside. */
__device__ __forceinline__ bool shapeHolds(const QShape &s, double cx, double cy, double cz, double side)
{
  const double h = side / 2;
  bool all = true;
  for (int n = 0; n < 8 && all; n++)
    all = shapeIn(s, (n & 1) ? cx + h : cx - h, (n & 2) ? cy + h : cy - h, (n & 4) ? cz + h : cz - h);
  return all;
}

/* mode 0: meet[l] = whether leaf l meets the shape (findBlocks);
 * mode 1: cnt[l] = points of leaf l that pointsIn returns;
 * mode 2: those points' record indices written from out + off[l]. */
template <int MODE>
__global__ void leafQueryKernel(QArgs a, uint32_t *__restrict__ cnt, const uint32_t *__restrict__ off,
                                uint32_t *__restrict__ out)
{
  const int lane = threadIdx.x & 31;
  const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t l = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; l < a.L; l += warps)
  {
    double cx, cy, cz, side;
    wb_leaf_cube(a.leafKey[l], a.leafLev[l], a.rootLo, a.rootSide, cx, cy, cz, side);
    const bool meets = shapeMeets(a.s, cx, cy, cz, side);
    if (MODE == 0)
    {
      if (lane == 0)
        cnt[l] = meets ? 1u : 0u;
      continue;
    }
    const uint32_t f = a.first[l], n = a.count[l];
    if (!meets)
    {
      if (MODE == 1 && lane == 0)
        cnt[l] = 0;
      continue;
    }
    const bool whole = shapeHolds(a.s, cx, cy, cz, side);
    uint32_t taken = 0;
    for (uint32_t t0 = 0; t0 < n; t0 += 32)
    {
      const uint32_t t = t0 + lane;
      bool in = false;
      if (t < n)
      {
        const uint32_t j = f + t;
        in = whole || shapeIn(a.s, wb_decode(a.sx[j], a.off[0], a.scale[0], a.unit),
                              wb_decode(a.sy[j], a.off[1], a.scale[1], a.unit),
                              wb_decode(a.sz[j], a.off[2], a.scale[2], a.unit));
      }
      const unsigned b = __ballot_sync(0xffffffffu, in);
      if (MODE == 2 && in)
        out[off[l] + taken + __popc(b & ((1u << lane) - 1))] = a.sidx[f + t];
      taken += __popc(b);
    }
    if (MODE == 1 && lane == 0)
      cnt[l] = taken;
  }
}

/* Order-preserving key of the height of record i (decoded), for the sort. */
__global__ void heightKeyKernel(uint64_t m, const uint32_t *__restrict__ recIdx, const uint32_t *__restrict__ storeOf,
                                const int32_t *__restrict__ sz, double off, double scale, double unit,
                                uint64_t *__restrict__ key, uint32_t *__restrict__ val)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
  {
    double z = wb_decode(sz[storeOf[recIdx[i]]], off, scale, unit);
    if (z == 0)
      z = 0;   // -0 and +0 compare equal
    uint64_t u;
    memcpy(&u, &z, 8);
    key[i] = (u >> 63) ? ~u : (u | 0x8000000000000000ull);
    val[i] = recIdx[i];
  }
}

__global__ void compactFlags(uint64_t L, const uint32_t *__restrict__ flag, const uint32_t *__restrict__ ex,
                             int64_t *__restrict__ out)
{
  for (uint64_t l = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; l < L; l += (uint64_t)gridDim.x * blockDim.x)
    if (flag[l])
      out[ex[l]] = (int64_t)l;
}

int shapeArgs(wb_ctx *c, const wb_shape *sh, QArgs &a, const char *who)
{
  if (!sh)
    return wb_fail(c, WB_EINVAL, std::string(who) + ": shape is NULL");
  memset(&a, 0, sizeof a);
  a.s.kind = sh->kind;
  if (sh->kind == WB_SHAPE_CYLINDER)
  {
    if (!(sh->r >= 0))
      return wb_fail(c, WB_EINVAL, std::string(who) + ": cylinder radius must be >= 0");
    a.s.cx = sh->v[0];
    a.s.cy = sh->v[1];
    a.s.r = sh->r;
  }
  else if (sh->kind == WB_SHAPE_HYPERBOLOID)
  {
    // Hyperboloid(v, r, s): por = r*s^2, centre = v + (0, 0, por) (shape.cpp:119-125)
    const double por = sh->r * (sh->s * sh->s);
    a.s.por2 = por * por;
    a.s.slope = sh->s;
    a.s.cx = sh->v[0] + 0;
    a.s.cy = sh->v[1] + 0;
    a.s.cz = sh->v[2] + por;
  }
  else
    return wb_fail(c, WB_EINVAL, std::string(who) + ": unknown shape kind");
  if (c->stage < 1)
    return wb_fail(c, WB_ESTATE, std::string(who) + ": no octree built");
  a.L = c->n_leaves;
  a.leafKey = (const uint64_t *)c->leafKey.p;
  a.leafLev = (const uint8_t *)c->leafLevel.p;
  a.first = (const uint32_t *)c->leafFirst.p;
  a.count = (const uint32_t *)c->leafCount.p;
  a.sx = (const int32_t *)c->sx.p;
  a.sy = (const int32_t *)c->sy.p;
  a.sz = (const int32_t *)c->sz.p;
  a.sidx = (const uint32_t *)c->sidx.p;
  for (int k = 0; k < 3; k++)
  {
    a.rootLo[k] = c->g.root_lo[k];
    a.off[k] = c->g.off[k];
    a.scale[k] = c->g.scale[k];
  }
  a.rootSide = c->g.root_side;
  a.unit = c->g.unit;
  return 0;
}

unsigned warpGrid(wb_ctx *c, uint64_t L)
{
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((L * 32 + 255) / 256, (uint64_t)c->sm_count * 32));
}
}  // namespace

extern "C" int wb_find_blocks(wb_ctx *c, const wb_shape *sh, int64_t *leaves, uint64_t capacity, uint64_t *count)
{
  if (!c || (capacity && !leaves))
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  QArgs a;
  int rc = shapeArgs(c, sh, a, "wb_find_blocks");
  if (rc)
    return rc;
  if (count)
    *count = 0;
  const uint64_t L = a.L;
  if (L == 0)
    return 0;
  WbScratch flag(c), ex(c), outD(c);
  if ((rc = wb_ensure(c, flag.b, L * 4 + 64)) || (rc = wb_ensure(c, ex.b, L * 4 + 64)) ||
      (rc = wb_ensure(c, outD.b, L * 8 + 64)))
    return rc;
  uint32_t *dTot = (uint32_t *)((uint8_t *)ex.b.p + L * 4);
  { leafQueryKernel<0><<<warpGrid(c, L), 256, 0, c->stream>>>(a, (uint32_t *)flag.b.p, nullptr, nullptr); ++c->launches; }
  if ((rc = wb_exclusive_scan_u32(c, (const uint32_t *)flag.b.p, (uint32_t *)ex.b.p, L, dTot)))
    return rc;
  uint32_t total = 0;
  WB_CUDA(c, cudaMemcpyAsync(&total, dTot, 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (count)
    *count = total;
  if (total > capacity)
    return wb_fail(c, WB_EINVAL, "wb_find_blocks: " + std::to_string(total) + " blocks, capacity " +
                                     std::to_string(capacity));
  { compactFlags<<<(unsigned)std::min<uint64_t>((L + 255) / 256, (uint64_t)c->sm_count * 16), 256, 0, c->stream>>>(
        L, (const uint32_t *)flag.b.p, (const uint32_t *)ex.b.p, (int64_t *)outD.b.p); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  if (total)
    WB_CUDA(c, cudaMemcpyAsync(leaves, outD.b.p, (size_t)total * 8, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  return 0;
}

extern "C" int wb_points_in(wb_ctx *c, const wb_shape *sh, int sorted, uint32_t *records, uint64_t capacity,
                            uint64_t *count)
{
  if (!c || (capacity && !records))
    return WB_EINVAL;
  WbDeviceGuard deviceGuard(c->device);
  QArgs a;
  int rc = shapeArgs(c, sh, a, "wb_points_in");
  if (rc)
    return rc;
  if (count)
    *count = 0;
  const uint64_t L = a.L;
  if (L == 0)
    return 0;
  WbScratch cnt(c), ex(c);
  if ((rc = wb_ensure(c, cnt.b, L * 4 + 64)) || (rc = wb_ensure(c, ex.b, L * 4 + 64)))
    return rc;
  uint32_t *dTot = (uint32_t *)((uint8_t *)ex.b.p + L * 4);
  { leafQueryKernel<1><<<warpGrid(c, L), 256, 0, c->stream>>>(a, (uint32_t *)cnt.b.p, nullptr, nullptr); ++c->launches; }
  if ((rc = wb_exclusive_scan_u32(c, (const uint32_t *)cnt.b.p, (uint32_t *)ex.b.p, L, dTot)))
    return rc;
  uint32_t total = 0;
  WB_CUDA(c, cudaMemcpyAsync(&total, dTot, 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (count)
    *count = total;
  if (total > capacity)
    return wb_fail(c, WB_EINVAL, "wb_points_in: " + std::to_string(total) + " points, capacity " +
                                     std::to_string(capacity));
  if (total == 0)
    return 0;
  WbScratch outD(c);
  if ((rc = wb_ensure(c, outD.b, (uint64_t)total * 4 + 64)))
    return rc;
  { leafQueryKernel<2><<<warpGrid(c, L), 256, 0, c->stream>>>(a, nullptr, (const uint32_t *)ex.b.p,
                                                             (uint32_t *)outD.b.p); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  const uint32_t *res = (const uint32_t *)outD.b.p;
  WbScratch k0(c), k1(c), v1(c);
  if (sorted && total > 1)
  {
    if ((rc = wb_ensure(c, k0.b, (uint64_t)total * 8 + 64)) || (rc = wb_ensure(c, k1.b, (uint64_t)total * 8 + 64)) ||
        (rc = wb_ensure(c, v1.b, (uint64_t)total * 4 + 64)))
      return rc;
    // the values are the record indices themselves; sort them by height in place of outD
    uint32_t *v0 = (uint32_t *)outD.b.p;
    { heightKeyKernel<<<(unsigned)std::min<uint64_t>((total + 255) / 256, (uint64_t)c->sm_count * 16), 256, 0,
                        c->stream>>>(total, v0, (const uint32_t *)c->storeOf.p, a.sz, a.off[2], a.scale[2], a.unit,
                                     (uint64_t *)k0.b.p, v0); ++c->launches; }
    uint64_t *keys = (uint64_t *)k0.b.p;
    uint32_t *vals = v0;
    if ((rc = wb_radix_sort_pairs(c, keys, vals, (uint64_t *)k1.b.p, (uint32_t *)v1.b.p, total, 0, 64)))
      return rc;
    res = vals;
  }
  WB_CUDA(c, cudaMemcpyAsync(records, res, (size_t)total * 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  return 0;
}

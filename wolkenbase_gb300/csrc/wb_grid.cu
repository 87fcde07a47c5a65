/* Column grid over the point store, the spatial index of the tile gather and
 * of classify.
 *
 * The reference answers every neighbourhood query by descending the octree
 * (Octree::findBlocks, octree.cpp:234-251).  Both queries of this path are
 * vertical: a cylinder (any z) and a downward hyperboloid whose horizontal
 * reach grows with depth.  A 2-D grid of square columns answers them with
 * plain ring walks: cells are visited outward from the query axis, so the
 * directions a classify query collects spread around the point early and the
 * surround test can stop after a few rings.
 *
 * Cells hold store positions sorted by height (so a query can stop reading a
 * column once its points are above the hyperboloid), a copy of the points'
 * integer X/Y/Z in grid order for coalesced reads, and per-cell integer
 * bounds for pruning.  A point that
 * lies outside the octree root cube is flagged: the reference's queries treat
 * such points through their leaf's cube, and the kernels do the same for them.
 */
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>
#include "wb_internal.h"
#include "wb_device.cuh"

namespace
{
struct GridArgs
{
  uint64_t nd;
  double off[3], scale[3], unit;
  double x0, y0, cell;
  int nx, ny;
  double rootLo[3], rootHi[3];
  /* integer thresholds (thr = 1: the decode increases with the record integer
     on every axis): xb[0..nx], yb[0..ny], then the root cube's faces
     {x, y, z lo, x, y, z hi} */
  const long long *bounds;
  int thr;
  float colPerUnit[2];
};

/* Smallest record integer X in [-2^31, 2^31) with pred(X), for a predicate
 * that is false then true as X grows; 2^31 when it never holds. */
template <typename P>
__device__ long long firstTrue(P pred)
{
  long long lo = -2147483648LL, hi = 2147483648LL;   // pred(lo) false, pred(hi) taken as true
  if (pred(lo))
    return lo;
  while (hi - lo > 1)
  {
    const long long mid = lo + (hi - lo) / 2;
    if (pred(mid))
      hi = mid;
    else
      lo = mid;
  }
  return hi;
}

/* The record-integer thresholds of the column boundaries and the root cube's
 * faces, one thread each, found with the same FP64 arithmetic the per-point
 * tests use: with a decode that increases with X, floor((dec(X) - x0) / cell)
 * >= i exactly when X >= xb[i], and dec(X) < lo exactly when X < xlo. */
__global__ void gridBoundsKernel(GridArgs g, long long *__restrict__ bounds)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int nb = (g.nx + 1) + (g.ny + 1);
  if (t <= g.nx)
    bounds[t] = firstTrue([&](long long X) {
      return floor((wb_decode((int32_t)X, g.off[0], g.scale[0], g.unit) - g.x0) / g.cell) >= (double)t;
    });
  else if (t < nb)
  {
    const int i = t - (g.nx + 1);
    bounds[t] = firstTrue([&](long long X) {
      return floor((wb_decode((int32_t)X, g.off[1], g.scale[1], g.unit) - g.y0) / g.cell) >= (double)i;
    });
  }
  else if (t < nb + 6)
  {
    const int ax = (t - nb) % 3;
    const double lim = (t - nb) < 3 ? g.rootLo[ax] : g.rootHi[ax];
    bounds[t] = firstTrue([&](long long X) { return wb_decode((int32_t)X, g.off[ax], g.scale[ax], g.unit) >= lim; });
  }
}

/* Column of record integer X on an axis with thresholds b[0..n]: X lies in
 * [b[0], b[n]); a guess from the mean column width, then the thresholds. */
__device__ __forceinline__ int columnOf(const long long *__restrict__ b, int n, long long X, float perUnit)
{
  int k = (int)((float)(X - b[0]) * perUnit);
  k = min(max(k, 0), n - 1);
  while (k > 0 && X < b[k])
    k--;
  while (k < n - 1 && X >= b[k + 1])
    k++;
  return k;
}

__global__ void cellKernel(GridArgs g, const int32_t *__restrict__ sx, const int32_t *__restrict__ sy,
                           const int32_t *__restrict__ sz, uint64_t *__restrict__ key, uint32_t *__restrict__ val,
                           uint8_t *__restrict__ stray, unsigned long long *__restrict__ nStray,
                           int *__restrict__ ext, const double *__restrict__ xyzd, int2 *__restrict__ colOf)
{
  // record-integer extent of the points ({min x, y, z}, {max x, y, z})
  int mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < g.nd; j += (uint64_t)gridDim.x * blockDim.x)
  {
    const int q[3] = {sx[j], sy[j], sz[j]};
    for (int a = 0; a < 3; a++)
    {
      mn[a] = min(mn[a], q[a]);
      mx[a] = max(mx[a], q[a]);
    }
    // the point's column as the classify set-up needs it (unclamped, within
    // +-1e9), and clamped into the grid for the sort key; from the integer
    // thresholds where they apply, else in FP64
    int ci, cj;
    bool sxy, s;
    if (g.thr)
    {
      const long long *xb = g.bounds, *yb = g.bounds + g.nx + 1, *face = g.bounds + g.nx + g.ny + 2;
      const long long X = q[0], Y = q[1], Z = q[2];
      if (X >= xb[0] && X < xb[g.nx])
        ci = columnOf(xb, g.nx, X, g.colPerUnit[0]);
      else
        ci = (int)fmax(fmin(floor((xyzd[j] - g.x0) / g.cell), 1e9), -1e9);
      if (Y >= yb[0] && Y < yb[g.ny])
        cj = columnOf(yb, g.ny, Y, g.colPerUnit[1]);
      else
        cj = (int)fmax(fmin(floor((xyzd[g.nd + j] - g.y0) / g.cell), 1e9), -1e9);
      sxy = X < face[0] || Y < face[1] || X >= face[3] || Y >= face[4];
      s = sxy || Z < face[2] || Z >= face[5];
    }
    else
    {
      const double x = xyzd[j], y = xyzd[g.nd + j], z = xyzd[2 * g.nd + j];
      ci = (int)fmax(fmin(floor((x - g.x0) / g.cell), 1e9), -1e9);
      cj = (int)fmax(fmin(floor((y - g.y0) / g.cell), 1e9), -1e9);
      sxy = x < g.rootLo[0] || y < g.rootLo[1] || x >= g.rootHi[0] || y >= g.rootHi[1];
      s = sxy || z < g.rootLo[2] || z >= g.rootHi[2];
    }
    colOf[j] = make_int2(ci, cj);
    const int cx = min(max(ci, 0), g.nx - 1), cy = min(max(cj, 0), g.ny - 1);
    // column in the high 32 bits, height (order-preserving int32 -> uint32) below
    key[j] = (((uint64_t)cy * g.nx + cx) << 32) | (uint32_t)(q[2] ^ (int32_t)0x80000000);
    val[j] = (uint32_t)j;
    stray[j] = (uint8_t)((s ? 1 : 0) | (sxy ? 2 : 0));
    if (s)
      atomicAdd(nStray, 1ull);
  }
  for (int a = 0; a < 3; a++)
    for (int o = 16; o; o >>= 1)
    {
      mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 3; a++)
    {
      atomicMin(&ext[a], mn[a]);
      atomicMax(&ext[3 + a], mx[a]);
    }
}

__global__ void cellStartKernel(uint64_t nd, uint64_t ncell, const uint64_t *__restrict__ key,
                                uint32_t *__restrict__ start)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint64_t k = key[i] >> 32;
    uint64_t prev = i ? key[i - 1] >> 32 : (uint64_t)-1;
    if (i == 0)
      for (uint64_t c = 0; c <= k; c++)
        start[c] = 0;
    else if (k != prev)
      for (uint64_t c = prev + 1; c <= k; c++)
        start[c] = (uint32_t)i;
    if (i == nd - 1)
      for (uint64_t c = k + 1; c <= ncell; c++)
        start[c] = (uint32_t)nd;
  }
}

/* Gathers the points into column order as int4 {X, Y, Z, position} and
 * forms each column's record; one warp per column. */
__global__ void cellFillKernel(uint64_t ncell, const uint32_t *__restrict__ start, const uint32_t *__restrict__ pos,
                               const int32_t *__restrict__ sx, const int32_t *__restrict__ sy,
                               const int32_t *__restrict__ sz, const uint8_t *__restrict__ stray,
                               int4 *__restrict__ gpt, int4 *__restrict__ rec)
{
  uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (c >= ncell)
    return;
  uint32_t b = start[c], e = start[c + 1];
  int32_t mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
  bool xyStray = false;
  for (uint32_t i = b + lane; i < e; i += 32)
  {
    uint32_t j = pos[i];
    int32_t q[3] = {sx[j], sy[j], sz[j]};
    uint8_t st = stray[j];
    gpt[i] = make_int4(q[0], q[1], q[2], (int)(j | ((st & 1) ? 0x80000000u : 0u)));
    xyStray |= (st & 2) != 0;
    for (int a = 0; a < 3; a++)
    {
      mn[a] = min(mn[a], q[a]);
      mx[a] = max(mx[a], q[a]);
    }
  }
  for (int a = 0; a < 3; a++)
    for (int o = 16; o; o >>= 1)
    {
      mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  // a column holding a point outside the root cube in x or y is read in full
  unsigned any = __ballot_sync(0xffffffffu, xyStray);
  if (lane == 0)
  {
    rec[2 * c] = make_int4(mn[0], mn[1], mx[0], mx[1]);
    rec[2 * c + 1] = make_int4(mn[2], (int)b, (int)e, any ? 1 : 0);
  }
}

/* Column groups (the classify work items): a column of n points is
 * ceil(n / 32) groups of consecutive points. */
__global__ void groupCountKernel(uint64_t ncell, const int4 *__restrict__ rec, uint32_t *__restrict__ cnt)
{
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (uint64_t)gridDim.x * blockDim.x)
  {
    int4 r1 = rec[2 * c + 1];
    cnt[c] = ((uint32_t)(r1.z - r1.y) + 31) / 32;
  }
}

__global__ void groupFillKernel(uint64_t ncell, const int4 *__restrict__ rec, const uint32_t *__restrict__ first,
                                uint2 *__restrict__ groups)
{
  for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (uint64_t)gridDim.x * blockDim.x)
  {
    int4 r1 = rec[2 * c + 1];
    uint32_t g = first[c];
    for (uint32_t t = (uint32_t)r1.y; t < (uint32_t)r1.z; t += 32)
      groups[g++] = make_uint2((uint32_t)c, t);
  }
}

/* Record-integer extent of the cloud: out[0..2] minima, out[3..5] maxima. */
/* Records of each block of WB_SUPER x WB_SUPER columns (the column record
 * layout; begin/end unused). */
__global__ void superKernel(int nx, int ny, int snx, int sny, const int4 *__restrict__ rec, int4 *__restrict__ srec)
{
  uint64_t ns = (uint64_t)snx * sny;
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += (uint64_t)gridDim.x * blockDim.x)
  {
    int si = (int)(s % snx), sj = (int)(s / snx);
    int32_t mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[2] = {INT32_MIN, INT32_MIN};
    for (int dj = 0; dj < WB_SUPER; dj++)
      for (int di = 0; di < WB_SUPER; di++)
      {
        int i = si * WB_SUPER + di, j = sj * WB_SUPER + dj;
        if (i >= nx || j >= ny)
          continue;
        uint64_t c = (uint64_t)j * nx + i;
        int4 r0 = rec[2 * c], r1 = rec[2 * c + 1];
        if (r1.y == r1.z)
          continue;
        mn[0] = min(mn[0], r0.x);
        mn[1] = min(mn[1], r0.y);
        mx[0] = max(mx[0], r0.z);
        mx[1] = max(mx[1], r0.w);
        mn[2] = min(mn[2], r1.x);
      }
    srec[2 * s] = make_int4(mn[0], mn[1], mx[0], mx[1]);
    srec[2 * s + 1] = make_int4(mn[2], 0, 0, 0);
  }
}
}  // namespace

int wb_grid_impl(wb_ctx *c, double x0, double y0, double x1, double y1)
{
  uint64_t nd = c->nd;
  WbGeom &g = c->g;
  double w = fmax(x1 - x0, 1e-9), h = fmax(y1 - y0, 1e-9);
  // about grid_points points per occupied column, at most 2^24 columns
  double cell = sqrt(w * h * c->grid_points / (double)(nd ? nd : 1));
  double minCell = sqrt(w * h / (double)(1u << 24));
  if (cell < minCell)
    cell = minCell;
  int nx = (int)ceil(w / cell) + 1, ny = (int)ceil(h / cell) + 1;
  c->grid.x0 = x0;
  c->grid.y0 = y0;
  c->grid.cell = cell;
  c->grid.nx = nx;
  c->grid.ny = ny;
  uint64_t ncell = (uint64_t)nx * ny;
  c->grid.ncell = ncell;
  int rc;
  if ((rc = wb_ensure(c, c->gKey0, nd * 8 + 64)) || (rc = wb_ensure(c, c->gKey1, nd * 8 + 64)) ||
      (rc = wb_ensure(c, c->gVal0, nd * 4 + 64)) || (rc = wb_ensure(c, c->gVal1, nd * 4 + 64)) ||
      (rc = wb_ensure(c, c->stray, nd + 64)) || (rc = wb_ensure(c, c->cellStart, (ncell + 1) * 4 + 64)) ||
      (rc = wb_ensure(c, c->gpt, nd * 16 + 64)) || (rc = wb_ensure(c, c->cellRec, ncell * 32 + 64)) ||
      (rc = wb_ensure(c, c->colOf, nd * 8 + 64)))
    return rc;
  GridArgs a;
  a.nd = nd;
  for (int k = 0; k < 3; k++)
  {
    a.off[k] = g.off[k];
    a.scale[k] = g.scale[k];
    a.rootLo[k] = g.root_lo[k];
    a.rootHi[k] = g.root_lo[k] + g.root_side;
  }
  a.unit = g.unit;
  a.x0 = x0;
  a.y0 = y0;
  a.cell = cell;
  a.nx = nx;
  a.ny = ny;
  // integer thresholds where every axis decodes increasingly
  a.thr = 0;
  a.bounds = nullptr;
  if (g.scale[0] * g.unit > 0 && g.scale[1] * g.unit > 0 && g.scale[2] * g.unit > 0)
  {
    const int nb = (nx + 1) + (ny + 1) + 6;
    if ((rc = wb_ensure(c, c->gridBounds, (size_t)nb * 8 + 64)))
      return rc;
    a.thr = 1;
    a.bounds = (const long long *)c->gridBounds.p;
    a.colPerUnit[0] = (float)(g.scale[0] * g.unit / cell);
    a.colPerUnit[1] = (float)(g.scale[1] * g.unit / cell);
    { gridBoundsKernel<<<(unsigned)((nb + 127) / 128), 128, 0, c->stream>>>(a, (long long *)c->gridBounds.p); ++c->launches; }
  }
  unsigned long long *dStray = (unsigned long long *)((char *)c->small.p + 256);
  int *dExt = (int *)((char *)c->small.p + 512);
  static const int kExtInit[6] = {INT32_MAX, INT32_MAX, INT32_MAX, INT32_MIN, INT32_MIN, INT32_MIN};
  WB_CUDA(c, cudaMemsetAsync(dStray, 0, 8, c->stream));
  WB_CUDA(c, cudaMemcpyAsync(dExt, kExtInit, 24, cudaMemcpyDefault, c->stream));
  unsigned blocks = (unsigned)std::min<uint64_t>((nd + 255) / 256 + 1, (uint64_t)c->sm_count * 16);
  uint64_t *key = (uint64_t *)c->gKey0.p;
  uint32_t *val = (uint32_t *)c->gVal0.p;
  { cellKernel<<<blocks, 256, 0, c->stream>>>(a, (const int32_t *)c->sx.p, (const int32_t *)c->sy.p,
                                              (const int32_t *)c->sz.p, key, val, (uint8_t *)c->stray.p, dStray,
                                              dExt, (const double *)c->xyzd.p, (int2 *)c->colOf.p); ++c->launches; }
  int bits = 1;
  while ((1ull << bits) < ncell)
    bits++;
  if ((rc = wb_radix_sort_pairs(c, key, val, (uint64_t *)c->gKey1.p, (uint32_t *)c->gVal1.p, nd, 0, 32 + bits)))
    return rc;
  uint32_t *start = (uint32_t *)c->cellStart.p;
  { cellStartKernel<<<blocks, 256, 0, c->stream>>>(nd, ncell, key, start); ++c->launches; }
  { cellFillKernel<<<(unsigned)((ncell * 32 + 255) / 256), 256, 0, c->stream>>>(
        ncell, start, val, (const int32_t *)c->sx.p, (const int32_t *)c->sy.p, (const int32_t *)c->sz.p,
        (const uint8_t *)c->stray.p, (int4 *)c->gpt.p, (int4 *)c->cellRec.p); ++c->launches; }
  int snx = (nx + WB_SUPER - 1) / WB_SUPER, sny = (ny + WB_SUPER - 1) / WB_SUPER;
  c->grid.snx = snx;
  c->grid.sny = sny;
  uint64_t nsup = (uint64_t)snx * sny;
  if ((rc = wb_ensure(c, c->superRec, nsup * 32 + 64)))
    return rc;
  { superKernel<<<(unsigned)std::min<uint64_t>((nsup + 255) / 256, (uint64_t)c->sm_count * 16), 256, 0, c->stream>>>(
        nx, ny, snx, sny, (const int4 *)c->cellRec.p, (int4 *)c->superRec.p); ++c->launches; }
  // column groups: counts, their prefix, the list
  uint32_t *gTot = (uint32_t *)((char *)c->small.p + 640);
  if ((rc = wb_ensure(c, c->groupCnt, (ncell + 1) * 8 + 64)))
    return rc;
  uint32_t *gcnt = (uint32_t *)c->groupCnt.p, *gfirst = gcnt + ncell + 1;
  { groupCountKernel<<<(unsigned)std::min<uint64_t>((ncell + 255) / 256, (uint64_t)c->sm_count * 16), 256, 0, c->stream>>>(
        ncell, (const int4 *)c->cellRec.p, gcnt); ++c->launches; }
  if ((rc = wb_exclusive_scan_u32(c, gcnt, gfirst, ncell, gTot)))
    return rc;
  // at most nd / 32 + ncell groups
  if ((rc = wb_ensure(c, c->groups, (nd / 32 + ncell + 1) * 8 + 64)))
    return rc;
  { groupFillKernel<<<(unsigned)std::min<uint64_t>((ncell + 255) / 256, (uint64_t)c->sm_count * 16), 256, 0, c->stream>>>(
        ncell, (const int4 *)c->cellRec.p, gfirst, (uint2 *)c->groups.p); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  unsigned long long ns = 0;
  uint32_t ngroups = 0;
  int ext[6];
  WB_CUDA(c, cudaMemcpyAsync(&ns, dStray, 8, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaMemcpyAsync(ext, dExt, 24, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaMemcpyAsync(&ngroups, gTot, 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  c->grid.nGroups = ngroups;
  c->grid.nStray = ns;
  c->grid.zminInt = ext[2];
  for (int k = 0; k < 3; k++)
  {
    c->grid.imin[k] = ext[k];
    c->grid.imax[k] = ext[3 + k];
  }
  return 0;
}

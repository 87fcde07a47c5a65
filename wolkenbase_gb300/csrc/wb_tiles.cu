/* Tile stage on the GPU: cylinder gathers, scanCylinder and postscanCylinder.
 *
 * Tile cylinders (Flowsnake::cyl, flowsnake.cpp:263-271) are gathered by one
 * warp per tile walking the node hierarchy depth-first in child order 0..7,
 * which visits leaves in the order Octree::findBlocks lists blocks; inside a
 * leaf, points are taken in store order.  That is the order
 * OctStore::pointsIn returns (octree.cpp:1214-1242) when each block holds its
 * points in input order, so the per-tile sums below are formed in the same
 * sequence as the reference's and the plane fit, the untilt and the
 * "second lowest" point come out identical.
 *
 * Pass 1 bounds each tile's points by the columns its cylinder meets (room
 * at tileStart[k]), pass 2 gathers them (tilePts from tileStart[k], tileN[k]
 * points) and records for every point the last tile in flowsnake order that
 * contains it (owner), which is the tile whose classification survives.
 */
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>
#include "wb_internal.h"
#include "wb_device.cuh"

namespace
{
constexpr int kTileWarps = 4;

struct TileArgs
{
  const int32_t *ex, *ey;
  uint64_t T;
  double cx, cy, spacing, rad;
  double off[3], scale[3], unit;
  const int32_t *child, *nodeBox, *leafBox;
  uint64_t N, L;
  const uint32_t *leafFirst, *leafCount;
  const uint64_t *leafKey;
  const uint8_t *leafLev;
  double rootLo[3], rootSide;
  const int32_t *sx, *sy, *sz;
  const double *xyzd;   /* decoded x, y, z planes of nd doubles */
  uint64_t nd;
  int fast;   /* FP32 filter allowed: decode steps nonzero (either sign), 32-bit record differences exact */
};

__device__ __forceinline__ void tileCenter(const TileArgs &a, uint64_t k, double &x, double &y)
{
  int e1 = a.ex[k], e2 = a.ey[k];
  double re = ((double)e1 - (double)e2 / 2.) * a.spacing;
  double im = ((double)e2 * 0.86602540378443864676372317) * a.spacing;
  x = re + a.cx;
  y = im + a.cy;
}

__device__ __forceinline__ double dec(const TileArgs &a, int ax, int32_t q)
{
  return wb_decode(q, a.off[ax], a.scale[ax], a.unit);
}

struct GridDev
{
  double x0, y0, cell;
  int nx, ny;
  const int4 *cell2;   /* two int4 per column: {x0, y0, x1, y1}, {zmin, begin, end, flags} */
  uint64_t ncell;
  const int4 *gpt;     /* int4 {X, Y, Z, position | stray bit} per point, column order */
  const uint32_t *leafId;
};

/* Cylinder::in for one point, exactly as the reference evaluates it; points
 * outside the root cube go through their leaf cube as OctStore::pointsIn
 * does (findBlocks test on the cube, all-corners fast path). */
__device__ bool cylExact(const TileArgs &a, const GridDev &gd, double cx, double cy, uint32_t gp, int32_t qx, int32_t qy)
{
  double px = dec(a, 0, qx), py = dec(a, 1, qy);
  bool in = wb_hypot(cx - px, cy - py) <= a.rad;
  if (!(gp & 0x80000000u))
    return in;
  uint32_t l = gd.leafId[gp & 0x7fffffffu];
  double lx, ly, lz, ls;
  wb_leaf_cube(a.leafKey[l], a.leafLev[l], a.rootLo, a.rootSide, lx, ly, lz, ls);
  if (!(wb_hypot(cx - wb_clamp_toward(cx, lx, ls), cy - wb_clamp_toward(cy, ly, ls)) <= a.rad))
    return false;
  bool all = true;
  for (int n = 0; n < 4; n++)
    all = all && wb_hypot(cx - ((n & 1) ? lx + ls / 2 : lx - ls / 2), cy - ((n & 2) ? ly + ls / 2 : ly - ls / 2)) <= a.rad;
  return all || in;
}

struct TileFrame
{
  double cx, cy;        /* cylinder centre (doubles, as Flowsnake::cyl)     */
  int32_t qx0, qy0;     /* integer part of the centre in record units       */
  float fx, fy;         /* fractional part                                  */
  float sx, sy;         /* metres per record unit                           */
  float r2lo, r2hi;     /* squared radius band that needs the exact test    */
  int i0, i1, j0, j1;   /* grid cells covering the cylinder                 */
};

__device__ TileFrame tileFrame(const TileArgs &a, const GridDev &gd, uint64_t k)
{
  TileFrame f;
  tileCenter(a, k, f.cx, f.cy);
  double ux = (f.cx / a.unit - a.off[0]) / a.scale[0], uy = (f.cy / a.unit - a.off[1]) / a.scale[1];
  double fx = floor(ux), fy = floor(uy);
  f.qx0 = (int32_t)fmax(fmin(fx, 2147483647.0), -2147483648.0);
  f.qy0 = (int32_t)fmax(fmin(fy, 2147483647.0), -2147483648.0);
  f.fx = (float)(ux - fx);
  f.fy = (float)(uy - fy);
  f.sx = (float)(a.scale[0] * a.unit);
  f.sy = (float)(a.scale[1] * a.unit);
  float r2 = (float)(a.rad * a.rad);
  f.r2lo = r2 * (1 - 2e-5f);
  f.r2hi = r2 * (1 + 2e-5f);
  double r = a.rad * (1 + 1e-9) + 1e-9;
  f.i0 = max(0, min(gd.nx - 1, (int)floor((f.cx - r - gd.x0) / gd.cell)));
  f.i1 = max(0, min(gd.nx - 1, (int)floor((f.cx + r - gd.x0) / gd.cell)));
  f.j0 = max(0, min(gd.ny - 1, (int)floor((f.cy - r - gd.y0) / gd.cell)));
  f.j1 = max(0, min(gd.ny - 1, (int)floor((f.cy + r - gd.y0) / gd.cell)));
  return f;
}

/* Membership of one grid point: FP32 distance in a frame centred on the
 * cylinder decides everything outside a +-2e-5 band around the radius; the
 * band and points outside the root cube use the exact double test. */
__device__ __forceinline__ bool cylMember(const TileArgs &a, const GridDev &gd, const TileFrame &f, uint32_t gp,
                                          int32_t qx, int32_t qy)
{
  if ((gp & 0x80000000u) || !a.fast)
    return cylExact(a, gd, f.cx, f.cy, gp, qx, qy);
  float dx = ((float)(qx - f.qx0) - f.fx) * f.sx;
  float dy = ((float)(qy - f.qy0) - f.fy) * f.sy;
  float d2 = dx * dx + dy * dy;
  if (d2 < f.r2lo)
    return true;
  if (d2 > f.r2hi)
    return false;
  return cylExact(a, gd, f.cx, f.cy, gp, qx, qy);
}

__device__ __forceinline__ bool cellMeetsCyl(const TileArgs &a, const int4 &box, double cx, double cy)
{
  // a negative scale reverses the decoded box
  double x0 = dec(a, 0, box.x), x1 = dec(a, 0, box.z);
  double y0 = dec(a, 1, box.y), y1 = dec(a, 1, box.w);
  if (x0 > x1)
  {
    const double t = x0;
    x0 = x1;
    x1 = t;
  }
  if (y0 > y1)
  {
    const double t = y0;
    y0 = y1;
    y1 = t;
  }
  double dx = cx < x0 ? x0 - cx : (cx > x1 ? cx - x1 : 0.0);
  double dy = cy < y0 ? y0 - cy : (cy > y1 ? cy - y1 : 0.0);
  double r = a.rad * (1 + 1e-6) + 1e-6;
  return dx * dx + dy * dy <= r * r;
}

/* The same column test in the tile's FP32 frame, with the radius widened by
 * 2e-4 (relative) and 1e-4 (absolute, squared units): a superset of the FP64
 * test (the frame's rounding is about 1e-7 relative), so no column with a
 * member is skipped; an extra column only costs its points' tests.  The
 * bound and both fills use this one test, so a tile never gathers more
 * points than its bound counted. */
__device__ __forceinline__ bool cellMeets(const TileArgs &a, const TileFrame &f, const int4 &box)
{
  if (!a.fast)
    return cellMeetsCyl(a, box, f.cx, f.cy);
  const float ax = ((float)(box.x - f.qx0) - f.fx) * f.sx, bx = ((float)(box.z - f.qx0) - f.fx) * f.sx;
  const float ay = ((float)(box.y - f.qy0) - f.fy) * f.sy, by = ((float)(box.w - f.qy0) - f.fy) * f.sy;
  // a negative scale reverses the box's ends
  const float x0 = fminf(ax, bx), x1 = fmaxf(ax, bx), y0 = fminf(ay, by), y1 = fmaxf(ay, by);
  const float dx = x0 > 0 ? x0 : (x1 < 0 ? -x1 : 0.f);
  const float dy = y0 > 0 ? y0 : (y1 < 0 ? -y1 : 0.f);
  return dx * dx + dy * dy <= f.r2hi * 1.0002f + 1e-8f;
}

/* Entries of the huge tiles as sort keys: (huge tile rank << 32) | store
 * position, huge tile h owning entries [pre[h], pre[h+1]). */
__global__ void hugeKeysKernel(uint32_t nh, const uint32_t *__restrict__ hugeList, const uint32_t *__restrict__ tileStart,
                               const uint64_t *__restrict__ pre, const uint32_t *__restrict__ tilePts,
                               uint64_t *__restrict__ keys, uint32_t *__restrict__ vals)
{
  const uint64_t total = pre[nh];
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t lo = 0, hi = nh;
    while (hi - lo > 1)
    {
      uint32_t mid = (lo + hi) >> 1;
      if (pre[mid] <= e)
        lo = mid;
      else
        hi = mid;
    }
    uint32_t base = tileStart[hugeList[lo]];
    keys[e] = ((uint64_t)lo << 32) | tilePts[base + (e - pre[lo])];
    vals[e] = 0;
  }
}

__global__ void hugeBackKernel(uint32_t nh, const uint32_t *__restrict__ hugeList, const uint32_t *__restrict__ tileStart,
                               const uint64_t *__restrict__ pre, const uint64_t *__restrict__ keys,
                               uint32_t *__restrict__ tilePts)
{
  const uint64_t total = pre[nh];
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t h = (uint32_t)(keys[e] >> 32);
    uint32_t base = tileStart[hugeList[h]];
    tilePts[base + (e - pre[h])] = (uint32_t)keys[e];
  }
}

/* Pass 1: one warp per tile counts the tile's points. */
/* Room for each tile's points: the points of the grid columns its cylinder
 * meets (an upper bound of the tile's count), one thread per tile.  The fill
 * passes write a tile's points from tileStart[k] on and its count to tileN. */
__global__ void gridBound(TileArgs a, GridDev gd, uint32_t *__restrict__ bound, TileFrame *__restrict__ frames)
{
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.T; k += (uint64_t)gridDim.x * blockDim.x)
  {
    const TileFrame f = tileFrame(a, gd, k);
    frames[k] = f;
    uint32_t room = 0;
    for (int j = f.j0; j <= f.j1; j++)
      for (int i = f.i0; i <= f.i1; i++)
      {
        uint64_t c = (uint64_t)j * gd.nx + i;
        int4 box = gd.cell2[2 * c], r1 = gd.cell2[2 * c + 1];
        if (r1.y != r1.z && cellMeets(a, f, box))
          room += (uint32_t)(r1.z - r1.y);
      }
    bound[k] = room;
  }
}

constexpr int kFillThreads = 256;
constexpr int kFillMax = 4096;

constexpr int kWarpFill = 1024;

/* Pass 2: one warp per tile gathers the tile's store positions, sorts them
 * (= OctStore::pointsIn order: leaf depth-first, then store order) with a
 * bitonic network in shared memory, and records each point's owner tile.
 * Tiles above kWarpFill points are listed for the block-wide version. */
__global__ void __launch_bounds__(32 * kTileWarps) gridFillWarp(TileArgs a, GridDev gd,
                                                                const uint32_t *__restrict__ tileStart,
                                                                uint32_t *__restrict__ tileN,
                                                                uint32_t *__restrict__ tilePts, int32_t *__restrict__ owner,
                                                                uint32_t *__restrict__ bigList, uint32_t *__restrict__ bigCount,
                                                                const TileFrame *__restrict__ frames)
{
  __shared__ uint32_t buf[kTileWarps][kWarpFill];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint64_t k = (uint64_t)blockIdx.x * kTileWarps + w;
  if (k >= a.T)
    return;
  const uint32_t base = tileStart[k];
  if (tileStart[k + 1] == base)
  {
    if (lane == 0)
      tileN[k] = 0;
    return;
  }
  uint32_t *b = buf[w];
  const unsigned lt = (1u << lane) - 1;
  const TileFrame f = frames[k];
  uint32_t n = 0;
  for (int j = f.j0; j <= f.j1; j++)
    for (int i = f.i0; i <= f.i1; i++)
    {
      uint64_t c = (uint64_t)j * gd.nx + i;
      int4 box = gd.cell2[2 * c], r1 = gd.cell2[2 * c + 1];
      uint32_t cb = (uint32_t)r1.y, ce = (uint32_t)r1.z;
      if (cb == ce || !cellMeets(a, f, box))
        continue;
      for (uint32_t t0 = cb; t0 < ce; t0 += 32)
      {
        uint32_t t = t0 + lane;
        uint32_t gp = 0;
        bool in = false;
        if (t < ce)
        {
          int4 p = gd.gpt[t];
          gp = (uint32_t)p.w;
          in = cylMember(a, gd, f, gp, p.x, p.y);
        }
        unsigned m = __ballot_sync(0xffffffffu, in);
        if (in && n + __popc(m & lt) < kWarpFill)
          b[n + __popc(m & lt)] = gp & 0x7fffffffu;
        n += __popc(m);
      }
    }
  const uint32_t M = n;
  if (lane == 0)
    tileN[k] = M;
  if (M == 0)
    return;
  if (M > kWarpFill)
  {
    // too many for the warp's buffer: the block-wide fill gathers it again
    if (lane == 0)
      bigList[atomicAdd(bigCount, 1u)] = (uint32_t)k;
    return;
  }
  int P = 32;
  while (P < (int)M)
    P <<= 1;
  for (int t = lane + (int)M; t < P; t += 32)
    b[t] = 0xffffffffu;
  __syncwarp();
  for (int kk = 2; kk <= P; kk <<= 1)
    for (int jj = kk >> 1; jj > 0; jj >>= 1)
    {
      for (int t = lane; t < P; t += 32)
      {
        int u = t ^ jj;
        if (u > t)
        {
          bool up = (t & kk) == 0;
          uint32_t x = b[t], y = b[u];
          if ((x > y) == up)
          {
            b[t] = y;
            b[u] = x;
          }
        }
      }
      __syncwarp();
    }
  for (uint32_t t = lane; t < M; t += 32)
  {
    uint32_t jpos = b[t];
    tilePts[base + t] = jpos;
    atomicMax(&owner[jpos], (int32_t)k);
  }
}

/* The block-wide fill for the tiles gridFillWarp listed: sorted in shared
 * memory up to kFillMax points; larger tiles are written unsorted, listed in
 * hugeList (*overflow counts them) and sorted by sortHugeTiles. */
__global__ void __launch_bounds__(kFillThreads) gridFill(TileArgs a, GridDev gd, const uint32_t *__restrict__ tileStart,
                                                         const uint32_t *__restrict__ tileN,
                                                         uint32_t *__restrict__ tilePts, int32_t *__restrict__ owner,
                                                         int *__restrict__ overflow, const uint32_t *__restrict__ bigList,
                                                         const uint32_t *__restrict__ bigCount,
                                                         uint32_t *__restrict__ hugeList,
                                                         const TileFrame *__restrict__ frames)
{
  __shared__ uint32_t buf[kFillMax];
  __shared__ uint32_t cnt;
  for (uint32_t bi = blockIdx.x; bi < *bigCount; bi += gridDim.x)
  {
  uint64_t k = bigList[bi];
  uint32_t base = tileStart[k], M = tileN[k];
  const bool huge = M > kFillMax;
  if (threadIdx.x == 0)
  {
    cnt = 0;
    // tiles above kFillMax points are written unsorted and sorted afterwards
    if (huge)
      hugeList[atomicAdd(overflow, 1)] = (uint32_t)k;
  }
  __syncthreads();
  const TileFrame f = frames[k];
  for (int j = f.j0; j <= f.j1; j++)
    for (int i = f.i0; i <= f.i1; i++)
    {
      uint64_t c = (uint64_t)j * gd.nx + i;
      int4 box = gd.cell2[2 * c], r1 = gd.cell2[2 * c + 1];
      uint32_t b = (uint32_t)r1.y, e = (uint32_t)r1.z;
      if (b == e || !cellMeets(a, f, box))
        continue;
      for (uint32_t t = b + threadIdx.x; t < e; t += kFillThreads)
      {
        int4 p = gd.gpt[t];
        uint32_t gp = (uint32_t)p.w;
        if (cylMember(a, gd, f, gp, p.x, p.y))
        {
          uint32_t slot = atomicAdd(&cnt, 1u);
          if (huge)
          {
            if (slot < M)
            {
              tilePts[base + slot] = gp & 0x7fffffffu;
              atomicMax(&owner[gp & 0x7fffffffu], (int32_t)k);
            }
          }
          else if (slot < kFillMax)
            buf[slot] = gp & 0x7fffffffu;
        }
      }
    }
  __syncthreads();
  if (huge)
    continue;
  int P = 1;
  while (P < (int)M)
    P <<= 1;
  for (int t = threadIdx.x + M; t < P; t += kFillThreads)
    buf[t] = 0xffffffffu;
  __syncthreads();
  for (int kk = 2; kk <= P; kk <<= 1)
    for (int jj = kk >> 1; jj > 0; jj >>= 1)
    {
      for (int t = threadIdx.x; t < P; t += kFillThreads)
      {
        int u = t ^ jj;
        if (u > t)
        {
          bool up = (t & kk) == 0;
          uint32_t x = buf[t], y = buf[u];
          if ((x > y) == up)
          {
            buf[t] = y;
            buf[u] = x;
          }
        }
      }
      __syncthreads();
    }
  for (uint32_t t = threadIdx.x; t < M; t += kFillThreads)
  {
    uint32_t j = buf[t];
    tilePts[base + t] = j;
    atomicMax(&owner[j], (int32_t)k);
  }
  __syncthreads();
  }
}

/* ---- scanCylinder ---- */
struct ScanArgs
{
  TileArgs t;
  const uint32_t *tileStart, *tileN, *tilePts;   /* tile k: tilePts[tileStart[k] ...], tileN[k] points */
  double minH;
};

constexpr int kQ = 8;   // summed quantities: xx, yx, yy, x, y, xz, yz, z
constexpr int kScanCache = 224;   // tile points whose coordinates stay in shared memory
constexpr int kScanWarps = 6;     // tiles (one warp each) per block of the exact scan's sums and shape passes

__device__ __forceinline__ void counterMergeGroup(double *part, uint64_t i, double g)
{
  uint64_t carry = i ^ (i + 8);
  if (carry == 8)
    part[3] = g;
  else
  {
    part[3] += g;
    int lvl = 4;
    for (; carry >> (lvl + 1); lvl++)
      part[lvl] += part[lvl - 1];
    part[lvl] = part[lvl - 1];
  }
}

__device__ __forceinline__ void counterMergeOne(double *part, uint64_t i, double v)
{
  uint64_t carry = i ^ (i + 1);
  if (carry == 1)
    part[0] = v;
  else
  {
    part[0] += v;
    int lvl = 1;
    for (; carry >> (lvl + 1); lvl++)
      part[lvl] += part[lvl - 1];
    part[lvl] = part[lvl - 1];
  }
}

/* Partial sums of the binary counter: 24 levels cover tiles of up to 2^26
 * points. */
constexpr int kLevels = 24;

__device__ double pairwiseFinish(const double *part, uint64_t n)
{
  double s = 0;
  for (int i = 0; i < kLevels; i++)
    if ((n >> i) & 1)
      s += part[i];
  return s;
}

/* 3x3 Gauss-Jordan with the reference's ratio pivoting (matrix.cpp:262-422). */
__device__ double pw3(double a, double b, double c)
{
  // pairwisesum of three values: ((a+b) + c) by the counter rule
  double part[4];
  part[0] = a;
  part[0] += b;
  part[1] = part[0];
  part[0] = c;
  double s = 0;
  s += part[0];
  s += part[1];
  return s;
}

__device__ double pwN(const double *v, int n)
{
  if (n == 1)
    return v[0];
  if (n == 2)
    return v[0] + v[1];
  return pw3(v[0], v[1], v[2]);
}

__device__ void swapRow(double m[3][3], double b[3], int r0, int r1)
{
  for (int k = 0; k < 3; k++)
  {
    double t = m[r0][k];
    m[r0][k] = m[r1][k];
    m[r1][k] = t;
  }
  double t = b[r0];
  b[r0] = b[r1];
  b[r1] = t;
}

__device__ void findPivot3(double m[3][3], double b[3], int row, int column)
{
  int pivotrow = -1;
  double maxratio = 0;
  for (; pivotrow < row && column < 3; column++)
    for (int i = row; i < 3; i++)
    {
      double sq[3] = {0, 0, 0};
      for (int j = column + 1; j < 3; j++)
        sq[j - column - 1] = m[i][j] * m[i][j];
      double ratio = (m[i][column] * m[i][column]) / pwN(sq, 3 - column);
      if (ratio > maxratio)
      {
        pivotrow = i;
        maxratio = ratio;
      }
    }
  if (pivotrow > row)
    swapRow(m, b, pivotrow, row);
}

__device__ void rowOp3(double m[3][3], double b[3], int row0, int row1, int piv)
{
  double slope = 0, minslope = INFINITY, det;
  int flags = 0, pivot;
  if (piv >= 0 && m[row0][piv] == 0 && m[row1][piv] == 0)
    piv = -1;
  pivot = piv;
  if (piv >= 0 && m[row0][piv] == 0)
    flags = 9;
  for (int i = 0; piv < 0 && i < 3; i++)
    if (m[row0][i] != 0 || m[row1][i] != 0)
    {
      if (fabs(m[row0][i]) > fabs(m[row1][i]) || row0 >= row1)
      {
        slope = fabs(m[row1][i] / m[row0][i]);
        flags &= ~8;
      }
      else
      {
        slope = fabs(m[row0][i] / m[row1][i]);
        flags |= 8;
      }
      if (slope < minslope)
      {
        minslope = slope;
        flags = (flags >> 3) * 9;
        pivot = i;
      }
    }
  flags &= 1;
  if (flags)
    swapRow(m, b, row0, row1);
  det = pivot < 0 ? 0 : m[row0][pivot];
  if (det != 0 && det != 1)
  {
    for (int i = 0; i < 3; i++)
      m[row0][i] /= det;
    b[row0] /= det;
  }
  if (pivot >= 0)
    slope = m[row1][pivot];
  if (slope != 0 && row0 != row1)
  {
    for (int i = 0; i < 3; i++)
      m[row1][i] -= m[row0][i] * slope;
    b[row1] -= b[row0] * slope;
  }
}

/* The histogram sector of a bottom point (scan.cpp:93-101): 0 inside the
 * inner circle hypot(x, y) < rin, else 1 + (rint(atan2(y, x) * 3 / pi) mod 6).
 * FP32 decides wherever it is at least 1e-5 (relative) away from the circle
 * and from a sector boundary (a half-integer of atan2 * 3 / pi); the rest is
 * evaluated in FP64 exactly as the reference writes it. */
__device__ __forceinline__ int sectorOf(double x, double y, double rin)
{
  const float xf = (float)x, yf = (float)y, rf = (float)rin;
  const float r2 = xf * xf + yf * yf, rin2 = rf * rf;
  bool inner;
  if (r2 < rin2 * (1 - 1e-5f))
    inner = true;
  else if (r2 > rin2 * (1 + 1e-5f))
    inner = false;
  else
    inner = wb_hypot(x, y) < rin;
  if (inner)
    return 0;
  const float v = atan2f(yf, xf) * 0.954929658551372f;   // 3 / pi
  const float half = floorf(v) + 0.5f;
  int sector;
  if (fabsf(v - half) > 1e-5f * (1.f + fabsf(v)))
    sector = (int)rintf(v);
  else
    sector = (int)rint(atan2(y, x) * 3 / M_PI);
  if (sector < 0)
    sector += 6;
  return (sector % 6) + 1;
}

/* scanCylinder in four kernels.  The FP64 pipe bounds this stage, and an
 * FP64 instruction costs the same whether one lane or 32 run it, so each part
 * runs at the width that keeps its lanes busy: the per-point passes one warp
 * per tile (lanes over points), everything done once per tile (centre, the
 * reference's 3x3 Gauss-Jordan, the slope clamp, density and height) one
 * thread per tile.  A tile's intermediate values live in one ScanWork slot;
 * its centre comes from the frame the gather's bound pass stored. */
union ScanWork
{
  double sums[kQ];   // scanSums -> scanSolve: the eight normal-equation sums
  struct
  {
    double sx, sy;          // scanSolve -> scanShape: the slope clamped to length 1
    double top, bottom;     // scanShape -> scanFinish
    uint32_t histo[7], nBottom;
  } s;
};

/* Pass 1: the eight sums of the normal equations that linearLeastSquares
 * forms from the tile's points (scan.cpp:60-68, matrix.cpp:194, 211) in the
 * reference's pairwise order (pairwisesum's binary counter over the points in
 * store order). */
__global__ void __launch_bounds__(32 * kScanWarps) scanSums(ScanArgs s, const TileFrame *__restrict__ frames,
                                                             ScanWork *__restrict__ work)
{
  __shared__ double part[kScanWarps][kQ][kLevels];
  __shared__ double tail[kScanWarps][kQ][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const TileArgs &a = s.t;
  const uint64_t k = (uint64_t)blockIdx.x * kScanWarps + w;
  if (k >= a.T)
    return;
  const uint32_t b0 = s.tileStart[k], M = s.tileN[k];
  if (M == 0)
    return;
  const double cx = frames[k].cx, cy = frames[k].cy;
  const uint64_t G = M / 8;   // complete groups of eight
  for (uint32_t c0 = 0; c0 < M; c0 += 32)
  {
    uint32_t i = c0 + lane;
    double q[kQ];
    if (i < M)
    {
      uint32_t j = s.tilePts[b0 + i];
      double x = a.xyzd[j] - cx, y = a.xyzd[a.nd + j] - cy, z = a.xyzd[2 * a.nd + j] - 0.0;
      q[0] = x * x;
      q[1] = y * x;
      q[2] = y * y;
      q[3] = 1.0 * x;
      q[4] = 1.0 * y;
      q[5] = x * z;
      q[6] = y * z;
      q[7] = 1.0 * z;
    }
    else
      for (int u = 0; u < kQ; u++)
        q[u] = 0;
    uint64_t grp = i / 8;
    // fixed tree inside each group of eight, ((a0+a1)+(a2+a3))+((a4+a5)+(a6+a7)),
    // for the eight quantities of the chunk's four groups: 224 additions in
    // seven FP64 instructions.  At each level a lane and its partner split
    // the quantities they both hold, so every lane's addition is a useful
    // one (addition commutes exactly; only the grouping is fixed).
    const bool l0 = lane & 1, l1 = (lane >> 1) & 1, l2 = (lane >> 2) & 1;
    double s1[4], s2[2], g;
#pragma unroll
    for (int r = 0; r < 4; r++)   // pairs: quantity 4*l0 + r
    {
      const double give = l0 ? q[r] : q[4 + r];
      s1[r] = (l0 ? q[4 + r] : q[r]) + __shfl_xor_sync(0xffffffffu, give, 1);
    }
#pragma unroll
    for (int t = 0; t < 2; t++)   // quads: quantity 4*l0 + 2*l1 + t
    {
      const double give = l1 ? s1[t] : s1[2 + t];
      s2[t] = (l1 ? s1[2 + t] : s1[t]) + __shfl_xor_sync(0xffffffffu, give, 2);
    }
    {                             // groups: quantity 4*l0 + 2*l1 + l2
      const double give = l2 ? s2[0] : s2[1];
      g = (l2 ? s2[1] : s2[0]) + __shfl_xor_sync(0xffffffffu, give, 4);
    }
    // lanes 0-7 merge their quantity for the up-to-4 complete groups of the
    // chunk, in group order (lane l + 8 gq holds group gq of the same quantity)
    const int uq = 4 * l0 + 2 * l1 + l2;
    for (int gq = 0; gq < 4; gq++)
    {
      const uint64_t gi = (uint64_t)c0 / 8 + gq;
      const double gv = __shfl_sync(0xffffffffu, g, (lane & 7) + 8 * gq);
      if (gi < G && lane < 8)
        counterMergeGroup(part[w][uq], gi * 8, gv);
    }
    // stash the trailing incomplete group's values
    if (i < M && grp == G)
      for (int u = 0; u < kQ; u++)
        tail[w][u][i - G * 8] = q[u];
    __syncwarp();
  }
  if (lane < kQ)
  {
    for (uint64_t i = G * 8; i < M; i++)
      counterMergeOne(part[w][lane], i, tail[w][lane][i - G * 8]);
    work[k].sums[lane] = pairwiseFinish(part[w][lane], M);
  }
}

/* The normal equations of each tile solved by one thread (matrix.cpp:262-422):
 * the plane goes into the tile's result, the slope clamped to length 1
 * (scan.cpp:69-73) into its work slot. */
__global__ void scanSolve(uint64_t T, const uint32_t *__restrict__ tileN, ScanWork *__restrict__ work,
                          TileRes *__restrict__ res)
{
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < T; k += (uint64_t)gridDim.x * blockDim.x)
  {
    const uint32_t M = tileN[k];
    if (M == 0)
      continue;
    double t[kQ];
    for (int u = 0; u < kQ; u++)
      t[u] = work[k].sums[u];
    double m[3][3] = {{t[0], t[1], t[3]}, {t[1], t[2], t[4]}, {t[3], t[4], (double)M}};
    double bv[3] = {t[5], t[6], t[7]};
    for (int i = 0; i < 3; i++)
    {
      findPivot3(m, bv, i, i);
      for (int j = 0; j < 3; j++)
        rowOp3(m, bv, i, j, i);
    }
    for (int i = 2; i >= 0; i--)
      for (int j = 0; j < i; j++)
        rowOp3(m, bv, i, j, i);
    const double v0 = m[0][0] == 0 ? NAN : bv[0], v1 = m[1][1] == 0 ? NAN : bv[1];
    res[k].plane[0] = v0;
    res[k].plane[1] = v1;
    res[k].plane[2] = m[2][2] == 0 ? NAN : bv[2];
    double sx = v0, sy = v1;
    const double len = wb_hypot(sx, sy);
    if (len > 1)
    {
      sx /= len;
      sy /= len;
    }
    if (isnan(sx) || isnan(sy))
      sx = sy = 0;
    work[k].s.sx = sx;
    work[k].s.sy = sy;
  }
}

/* Passes 2-4 of scanCylinder (scan.cpp:74-102): untilt by the clamped
 * slope, bottom (first minimum), bottom2 (minimum before it), top and the
 * sector histogram of the bottom points.  Each lane keeps its own minimum (with its first index), maximum
 * and bottom2 over its points and the warp combines them once per tile:
 * the first minimum is the least (height, index) pair whatever the order,
 * and fmin / fmax give the same value in any order (they order -0 below +0). */
__global__ void __launch_bounds__(32 * kScanWarps) scanShape(ScanArgs s, const TileFrame *__restrict__ frames,
                                                              ScanWork *__restrict__ work)
{
  // tile-local coordinates and untilted heights of tiles up to kScanCache
  // points, computed once
  __shared__ double cxy[kScanWarps][4][kScanCache];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const TileArgs &a = s.t;
  const uint64_t k = (uint64_t)blockIdx.x * kScanWarps + w;
  if (k >= a.T)
    return;
  const uint32_t b0 = s.tileStart[k], M = s.tileN[k];
  if (M == 0)
    return;
  const double cx = frames[k].cx, cy = frames[k].cy;
  const bool cached = M <= kScanCache;
  if (cached)
  {
    for (uint32_t i = lane; i < M; i += 32)
    {
      uint32_t j = s.tilePts[b0 + i];
      cxy[w][0][i] = a.xyzd[j] - cx;
      cxy[w][1][i] = a.xyzd[a.nd + j] - cy;
      cxy[w][2][i] = a.xyzd[2 * a.nd + j] - 0.0;
    }
    __syncwarp();
  }
  // coordinates of tile point i: from the cache, or decoded again
  auto coords = [&](uint32_t i, double &x, double &y, double &z) {
    if (cached)
    {
      x = cxy[w][0][i];
      y = cxy[w][1][i];
      z = cxy[w][2][i];
    }
    else
    {
      uint32_t j = s.tilePts[b0 + i];
      x = a.xyzd[j] - cx;
      y = a.xyzd[a.nd + j] - cy;
      z = a.xyzd[2 * a.nd + j] - 0.0;
    }
  };
  const double sx = work[k].s.sx, sy = work[k].s.sy;
  // untilted height of tile point i (cached tiles: from the cache once pass 2 stored it)
  auto untilted = [&](uint32_t i) -> double {
    if (cached)
      return cxy[w][3][i];
    double x, y, z;
    coords(i, x, y, z);
    return z - (sy * y + sx * x);
  };
  // untilt: bottom (first minimum), top
  double mv = INFINITY, top = -INFINITY;
  uint32_t mi = 0xffffffffu;
  for (uint32_t i = lane; i < M; i += 32)
  {
    double x, y, z;
    coords(i, x, y, z);
    const double uz = z - (sy * y + sx * x);
    if (cached)
      cxy[w][3][i] = uz;
    if (uz < mv)
    {
      mv = uz;
      mi = i;
    }
    top = fmax(top, uz);
  }
  for (int o = 16; o; o >>= 1)
  {
    const double ov = __shfl_xor_sync(0xffffffffu, mv, o);
    const uint32_t oi = __shfl_xor_sync(0xffffffffu, mi, o);
    if (ov < mv || (ov == mv && oi < mi))
    {
      mv = ov;
      mi = oi;
    }
    top = fmax(top, __shfl_xor_sync(0xffffffffu, top, o));
  }
  const double bottom = mv < INFINITY ? mv : INFINITY;
  const uint32_t argmin = mv < INFINITY ? mi : 0xffffffffu;
  __syncwarp();
  // bottom2: the lowest untilted height before the first minimum
  double bottom2 = INFINITY;
  for (uint32_t i = lane; i < M && i < argmin; i += 32)
    bottom2 = fmin(bottom2, untilted(i));
  for (int o = 16; o; o >>= 1)
    bottom2 = fmin(bottom2, __shfl_xor_sync(0xffffffffu, bottom2, o));
  if (isinf(bottom2))
    bottom2 = bottom;
  // sector histogram of the points within 2 rad of bottom2
  const double zcut = bottom2 + 2 * a.rad, rin = a.rad / 2.6457513110645905905016;
  uint32_t nBottom = 0;
  int histo[7] = {0, 0, 0, 0, 0, 0, 0};
  for (uint32_t c0 = 0; c0 < M; c0 += 32)
  {
    uint32_t i = c0 + lane;
    int sector = -1;
    if (i < M && untilted(i) < zcut)
    {
      double x, y, z;
      coords(i, x, y, z);
      sector = sectorOf(x, y, rin);
    }
    for (int sct = 0; sct < 7; sct++)
      histo[sct] += __popc(__ballot_sync(0xffffffffu, sector == sct));
    nBottom += __popc(__ballot_sync(0xffffffffu, sector >= 0));
  }
  if (lane == 0)
  {
    ScanWork &o = work[k];
    o.s.top = top;
    o.s.bottom = bottom;
    for (int i = 0; i < 7; i++)
      o.s.histo[i] = (uint32_t)histo[i];
    o.s.nBottom = nBottom;
  }
}

/* Density, tree flags, h and height of each tile (scan.cpp:103-120), one
 * thread per tile. */
__device__ __forceinline__ const ScanWork &asWork(const ScanWork &x)
{
  return x;
}

template <typename Slot>
__global__ void scanFinish(uint64_t T, const uint32_t *__restrict__ tileN, const Slot *__restrict__ work,
                           double rad, double minH, TileRes *__restrict__ res)
{
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < T; k += (uint64_t)gridDim.x * blockDim.x)
  {
    const uint32_t M = tileN[k];
    TileRes r{};
    if (M == 0)
    {
      res[k] = r;
      continue;
    }
    const ScanWork &o = asWork(work[k]);
    r.plane[0] = res[k].plane[0];
    r.plane[1] = res[k].plane[1];
    r.plane[2] = res[k].plane[2];
    double density = 0;
    int treeFlags = 0;
    for (int i = 0; i < 7; i++)
      density += (double)(int)o.s.histo[i] * (double)(int)o.s.histo[i];
    if (M > o.s.nBottom && density < 7)
      treeFlags = 1;
    density = sqrt(density) * 2.6457513110645905905016 / (rad * rad) / M_PI;
    if (M > o.s.nBottom && density < 0.5)
      treeFlags = 1;
    if (o.s.top - o.s.bottom > 1.5)
      treeFlags = 1;
    r.nPoints = (int32_t)M;
    r.nGround = 0;
    r.treeFlags = treeFlags;
    r.density = density;
    r.hScan = r.h = sqrt(1 / density + minH * minH);
    r.height = o.s.top - o.s.bottom;
    res[k] = r;
  }
}

/* Error-free sum of two floats (Knuth's two-sum): s + e == a + b exactly. */
__device__ __forceinline__ void twoSumF(float a, float b, float &s, float &e)
{
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

/* scanCylinder in the precision mode: coordinates are FP32 in a tile-local
 * frame (record integers minus an integer anchor next to the tile centre,
 * times the scale).  The normal-equation sums are taken about the points'
 * centroid in record integers, accumulated per lane with Kahan compensation
 * and merged across the warp with two-sums; the untilting, bottom, bottom2,
 * top and the sector histogram run in FP32 in the anchor frame.  As in the
 * exact mode, everything done once per tile runs one thread per tile: the
 * rebuild of the tile-centre sums in FP64, the 3x3 solve (the reference's
 * Gauss-Jordan with ratio pivoting), the slope clamp, density and height. */
struct Scan32Sums
{
  float hi[kQ], lo[kQ];       // compensated sums about the centroid, hi + lo
  int32_t cX, cY, cZ, az;     // centroid and the height anchor, record integers
};
union ScanWork32
{
  Scan32Sums p;   // scan32Sums -> scan32Solve
  ScanWork w;     // scan32Solve -> scan32Shape -> scanFinish (az stays in p)
};

__device__ __forceinline__ const ScanWork &asWork(const ScanWork32 &x)
{
  return x.w;
}

/* The tile-local FP32 frame: anchor (qx0, qy0) of the tile frame, the anchor's
 * offset from the centre in metres, heights from az. */
struct Frame32
{
  int32_t ax, ay, az;
  float fx, fy, ssx, ssy, ssz;
};

__device__ __forceinline__ Frame32 frame32(const TileArgs &a, const TileFrame &f, int32_t az)
{
  Frame32 g;
  g.ax = f.qx0;
  g.ay = f.qy0;
  g.az = az;
  g.ssx = f.sx;
  g.ssy = f.sy;
  g.ssz = (float)(a.scale[2] * a.unit);
  g.fx = -__fmul_rn(f.fx, f.sx);
  g.fy = -__fmul_rn(f.fy, f.sy);
  return g;
}

__device__ __forceinline__ void local32(const TileArgs &a, const Frame32 &g, uint32_t j, float &x, float &y, float &z)
{
  x = __fadd_rn(__fmul_rn((float)(a.sx[j] - g.ax), g.ssx), g.fx);
  y = __fadd_rn(__fmul_rn((float)(a.sy[j] - g.ay), g.ssy), g.fy);
  z = __fmul_rn((float)(a.sz[j] - g.az), g.ssz);
}

/* Pass 1 of the precision mode, one warp per tile: the centroid in record
 * integers (exact int64 sums) and the compensated sums of the products of
 * u = X - centroid (exact in FP32), which are exact while a product stays
 * below 2^24 (|u| * |v| of a 1.5 m tile at 1 mm is below 2^20). */
__global__ void __launch_bounds__(32 * kScanWarps) scan32Sums(ScanArgs s, ScanWork32 *__restrict__ work)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const TileArgs &a = s.t;
  const uint64_t k = (uint64_t)blockIdx.x * kScanWarps + w;
  if (k >= a.T)
    return;
  const uint32_t b0 = s.tileStart[k], M = s.tileN[k];
  if (M == 0)
    return;
  // the first point as the origin of the integer sums (the cloud spans less
  // than 2^30 record units, so the differences fit)
  const uint32_t j0 = s.tilePts[b0];
  const int32_t ox = a.sx[j0], oy = a.sy[j0], az = a.sz[j0];
  long long isum[3] = {0, 0, 0};
  for (uint32_t i = lane; i < M; i += 32)
  {
    const uint32_t j = s.tilePts[b0 + i];
    isum[0] += a.sx[j] - ox;
    isum[1] += a.sy[j] - oy;
    isum[2] += a.sz[j] - az;
  }
  for (int d = 0; d < 3; d++)
    for (int o = 16; o; o >>= 1)
      isum[d] += __shfl_xor_sync(0xffffffffu, isum[d], o);
  // an integer next to the centroid (truncated quotient): only the origin of
  // the FP32 products, so any nearby integer will do
  const int32_t cX = ox + (int32_t)(isum[0] / (long long)M), cY = oy + (int32_t)(isum[1] / (long long)M),
                cZ = az + (int32_t)(isum[2] / (long long)M);
  float sum[kQ], cmp[kQ];
  for (int u = 0; u < kQ; u++)
    sum[u] = cmp[u] = 0.f;
  for (uint32_t i = lane; i < M; i += 32)
  {
    const uint32_t j = s.tilePts[b0 + i];
    const float u = (float)(a.sx[j] - cX), v = (float)(a.sy[j] - cY), t = (float)(a.sz[j] - cZ);
    float q[kQ];
    q[0] = __fmul_rn(u, u);
    q[1] = __fmul_rn(v, u);
    q[2] = __fmul_rn(v, v);
    q[3] = u;
    q[4] = v;
    q[5] = __fmul_rn(u, t);
    q[6] = __fmul_rn(v, t);
    q[7] = t;
    for (int e = 0; e < kQ; e++)
    {
      const float yv = __fsub_rn(q[e], cmp[e]);
      const float tt = __fadd_rn(sum[e], yv);
      cmp[e] = __fsub_rn(__fsub_rn(tt, sum[e]), yv);
      sum[e] = tt;
    }
  }
  Scan32Sums out;
  for (int e = 0; e < kQ; e++)
  {
    float hi = sum[e], lo = -cmp[e];
    for (int o = 16; o; o >>= 1)
    {
      const float ohi = __shfl_xor_sync(0xffffffffu, hi, o), olo = __shfl_xor_sync(0xffffffffu, lo, o);
      float sh, se;
      twoSumF(hi, ohi, sh, se);
      hi = sh;
      lo = __fadd_rn(__fadd_rn(lo, olo), se);
    }
    out.hi[e] = hi;
    out.lo[e] = lo;
  }
  out.cX = cX;
  out.cY = cY;
  out.cZ = cZ;
  out.az = az;
  if (lane == 0)
    work[k].p = out;
}

/* The tile-centre sums rebuilt in FP64 from the centroid sums (x = u kx + X,
 * y = v ky + Y, z - z0 = t kz + Z), the solve and the slope clamp, one
 * thread per tile. */
__global__ void scan32Solve(TileArgs a, const uint32_t *__restrict__ tileN, const TileFrame *__restrict__ frames,
                            ScanWork32 *__restrict__ work, TileRes *__restrict__ res)
{
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < a.T; k += (uint64_t)gridDim.x * blockDim.x)
  {
    const uint32_t M = tileN[k];
    if (M == 0)
      continue;
    const Scan32Sums p = work[k].p;
    double cs[kQ];
    for (int e = 0; e < kQ; e++)
      cs[e] = (double)p.hi[e] + (double)p.lo[e];
    const double cx = frames[k].cx, cy = frames[k].cy, z0 = dec(a, 2, p.az);
    const double kx = a.scale[0] * a.unit, ky = a.scale[1] * a.unit, kz = a.scale[2] * a.unit;
    const double X = dec(a, 0, p.cX) - cx, Y = dec(a, 1, p.cY) - cy, Z = dec(a, 2, p.cZ) - z0, Md = (double)M;
    const double uu = cs[0] * kx * kx, uv = cs[1] * kx * ky, vv = cs[2] * ky * ky, su = cs[3] * kx, sv = cs[4] * ky,
                 ut = cs[5] * kx * kz, vt = cs[6] * ky * kz, st = cs[7] * kz;
    double tot[kQ];
    tot[0] = uu + 2 * X * su + Md * X * X;
    tot[1] = uv + X * sv + Y * su + Md * X * Y;
    tot[2] = vv + 2 * Y * sv + Md * Y * Y;
    tot[3] = su + Md * X;
    tot[4] = sv + Md * Y;
    tot[5] = ut + Z * su + X * st + Md * X * Z;
    tot[6] = vt + Z * sv + Y * st + Md * Y * Z;
    tot[7] = st + Md * Z;
    double m[3][3] = {{tot[0], tot[1], tot[3]}, {tot[1], tot[2], tot[4]}, {tot[3], tot[4], Md}};
    double bv[3] = {tot[5], tot[6], tot[7]};
    for (int i = 0; i < 3; i++)
    {
      findPivot3(m, bv, i, i);
      for (int j = 0; j < 3; j++)
        rowOp3(m, bv, i, j, i);
    }
    for (int i = 2; i >= 0; i--)
      for (int j = 0; j < i; j++)
        rowOp3(m, bv, i, j, i);
    const double v0 = m[0][0] == 0 ? NAN : bv[0], v1 = m[1][1] == 0 ? NAN : bv[1];
    res[k].plane[0] = v0;
    res[k].plane[1] = v1;
    res[k].plane[2] = m[2][2] == 0 ? NAN : bv[2] + z0;
    double sx = v0, sy = v1;
    const double len = wb_hypot(sx, sy);
    if (len > 1)
    {
      sx /= len;
      sy /= len;
    }
    if (isnan(sx) || isnan(sy))
      sx = sy = 0;
    work[k].w.s.sx = sx;
    work[k].w.s.sy = sy;
  }
}

/* Passes 2-4 of the precision mode, one warp per tile, in FP32: untilt,
 * bottom (first minimum), bottom2, top and the sector histogram. */
__global__ void __launch_bounds__(32 * kScanWarps) scan32Shape(ScanArgs s, const TileFrame *__restrict__ frames,
                                                               ScanWork32 *__restrict__ work)
{
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const TileArgs &a = s.t;
  const uint64_t k = (uint64_t)blockIdx.x * kScanWarps + w;
  if (k >= a.T)
    return;
  const uint32_t b0 = s.tileStart[k], M = s.tileN[k];
  if (M == 0)
    return;
  const Frame32 g = frame32(a, frames[k], work[k].p.az);
  const float fsx = (float)work[k].w.s.sx, fsy = (float)work[k].w.s.sy;
  auto untilt = [&](float x, float y, float z) { return __fsub_rn(z, __fadd_rn(__fmul_rn(fsy, y), __fmul_rn(fsx, x))); };
  float mv = INFINITY, top = -INFINITY;
  uint32_t mi = 0xffffffffu;
  for (uint32_t i = lane; i < M; i += 32)
  {
    float x, y, z;
    local32(a, g, s.tilePts[b0 + i], x, y, z);
    const float uz = untilt(x, y, z);
    if (uz < mv)
    {
      mv = uz;
      mi = i;
    }
    top = fmaxf(top, uz);
  }
  for (int o = 16; o; o >>= 1)
  {
    const float ov = __shfl_xor_sync(0xffffffffu, mv, o);
    const uint32_t oi = __shfl_xor_sync(0xffffffffu, mi, o);
    if (ov < mv || (ov == mv && oi < mi))
    {
      mv = ov;
      mi = oi;
    }
    top = fmaxf(top, __shfl_xor_sync(0xffffffffu, top, o));
  }
  const float bottom = mv;
  const uint32_t argmin = mi;
  float bottom2 = INFINITY;
  for (uint32_t i = lane; i < M && i < argmin; i += 32)
  {
    float x, y, z;
    local32(a, g, s.tilePts[b0 + i], x, y, z);
    bottom2 = fminf(bottom2, untilt(x, y, z));
  }
  for (int o = 16; o; o >>= 1)
    bottom2 = fminf(bottom2, __shfl_xor_sync(0xffffffffu, bottom2, o));
  if (isinf(bottom2))
    bottom2 = bottom;
  const float lim = __fadd_rn(bottom2, (float)(2 * a.rad)), inner = (float)(a.rad / 2.6457513110645905905016);
  uint32_t nBottom = 0;
  int histo[7] = {0, 0, 0, 0, 0, 0, 0};
  for (uint32_t c0 = 0; c0 < M; c0 += 32)
  {
    const uint32_t i = c0 + lane;
    int sector = -1;
    if (i < M)
    {
      float x, y, z;
      local32(a, g, s.tilePts[b0 + i], x, y, z);
      if (untilt(x, y, z) < lim)
      {
        sector = (int)rintf(atan2f(y, x) * 0.954929658551372f);   // 3 / pi
        if (sector < 0)
          sector += 6;
        sector = (sector % 6) + 1;
        if (hypotf(x, y) < inner)
          sector = 0;
      }
    }
    for (int sct = 0; sct < 7; sct++)
      histo[sct] += __popc(__ballot_sync(0xffffffffu, sector == sct));
    nBottom += __popc(__ballot_sync(0xffffffffu, sector >= 0));
  }
  if (lane == 0)
  {
    ScanWork &o = work[k].w;
    o.s.top = (double)top;
    o.s.bottom = (double)bottom;
    for (int e = 0; e < 7; e++)
      o.s.histo[e] = (uint32_t)histo[e];
    o.s.nBottom = nBottom;
  }
}

/* postscanCylinder (scan.cpp:142-179): tree tiles grow their hyperboloid by
 * the number of tree tiles met walking the six lattice rays. */
__global__ void postscanKernel(uint64_t T, const int32_t *__restrict__ ex, const int32_t *__restrict__ ey,
                               const int32_t *__restrict__ lookup, int x0, int y0, int W, int H, double spacing,
                               TileRes *__restrict__ res, double *__restrict__ hOut)
{
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < T; k += (uint64_t)gridDim.x * blockDim.x)
  {
    TileRes me = res[k];
    double h = me.h;
    if (me.nPoints)
    {
      const int rx[6] = {1, 1, 0, -1, -1, 0}, ry[6] = {0, 1, 1, 0, -1, -1};
      int i = 1, count = 0, nontree, ringcount;
      do
      {
        nontree = ringcount = 0;
        for (int j = 0; j < 6 && (me.treeFlags & 1); j++)
        {
          int ax = ex[k] + rx[j] * i - x0, ay = ey[k] + ry[j] * i - y0;
          if (ax < 0 || ay < 0 || ax >= W || ay >= H)
            continue;
          int32_t kk = lookup[(uint64_t)ay * W + ax];
          if (kk < 0)
            continue;
          TileRes o = res[kk];
          if (o.nPoints)
          {
            ringcount++;
            if (o.treeFlags & 1)
              count++;
            else
              nontree++;
          }
        }
        ++i;
      } while (ringcount && !nontree);
      double e = count * spacing / 6;
      h = sqrt(h * h + e * e);
    }
    hOut[k] = h;
  }
}

__global__ void applyH(uint64_t T, const double *__restrict__ hIn, TileRes *__restrict__ res)
{
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < T; k += (uint64_t)gridDim.x * blockDim.x)
    res[k].h = hIn[k];
}

__global__ void fillOwner(int32_t *p, uint64_t n)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = -1;
}
}  // namespace

static int uploadTiles(wb_ctx *c)
{
  WbGeom &g = c->g;
  if (c->flowIdxCached != g.snake_idx)
  {
    wb_flowsnake_order(g.snake_idx, c->flowHostEx, c->flowHostEy);
    uint64_t T = c->flowHostEx.size();
    int x0 = INT32_MAX, y0 = INT32_MAX, x1 = INT32_MIN, y1 = INT32_MIN;
    for (uint64_t k = 0; k < T; k++)
    {
      x0 = std::min(x0, c->flowHostEx[k]);
      x1 = std::max(x1, c->flowHostEx[k]);
      y0 = std::min(y0, c->flowHostEy[k]);
      y1 = std::max(y1, c->flowHostEy[k]);
    }
    c->lookupX0 = x0;
    c->lookupY0 = y0;
    c->lookupW = x1 - x0 + 1;
    c->lookupH = y1 - y0 + 1;
    std::vector<int32_t> look((uint64_t)c->lookupW * c->lookupH, -1);
    for (uint64_t k = 0; k < T; k++)
      look[(uint64_t)(c->flowHostEy[k] - y0) * c->lookupW + (c->flowHostEx[k] - x0)] = (int32_t)k;
    int rc;
    if ((rc = wb_ensure(c, c->tileEx, T * 4 + 64)) || (rc = wb_ensure(c, c->tileEy, T * 4 + 64)) ||
        (rc = wb_ensure(c, c->tileLookup, look.size() * 4 + 64)))
      return rc;
    WB_CUDA(c, cudaMemcpyAsync(c->tileEx.p, c->flowHostEx.data(), T * 4, cudaMemcpyDefault, c->stream));
    WB_CUDA(c, cudaMemcpyAsync(c->tileEy.p, c->flowHostEy.data(), T * 4, cudaMemcpyDefault, c->stream));
    WB_CUDA(c, cudaMemcpyAsync(c->tileLookup.p, look.data(), look.size() * 4, cudaMemcpyDefault, c->stream));
    WB_CUDA(c, cudaStreamSynchronize(c->stream));
    c->flowIdxCached = g.snake_idx;
  }
  c->n_tiles = c->flowHostEx.size();
  return 0;
}

static TileArgs tileArgs(wb_ctx *c)
{
  TileArgs a;
  WbGeom &g = c->g;
  a.ex = (const int32_t *)c->tileEx.p;
  a.ey = (const int32_t *)c->tileEy.p;
  a.T = c->n_tiles;
  a.cx = g.tile_c[0];
  a.cy = g.tile_c[1];
  a.spacing = g.spacing;
  a.rad = g.spacing * 41 / 71;
  for (int k = 0; k < 3; k++)
  {
    a.off[k] = g.off[k];
    a.scale[k] = g.scale[k];
  }
  a.unit = g.unit;
  a.child = (const int32_t *)c->nodeChild.p;
  a.nodeBox = (const int32_t *)c->nodeBox.p;
  a.leafBox = (const int32_t *)c->leafBox.p;
  a.N = c->n_nodes;
  a.L = c->n_leaves;
  a.leafFirst = (const uint32_t *)c->leafFirst.p;
  a.leafCount = (const uint32_t *)c->leafCount.p;
  a.leafKey = (const uint64_t *)c->leafKey.p;
  a.leafLev = (const uint8_t *)c->leafLevel.p;
  for (int k = 0; k < 3; k++)
    a.rootLo[k] = g.root_lo[k];
  a.rootSide = g.root_side;
  a.fast = 0;
  {
    // the centre's integer part stays within a tile of the cloud, so 32-bit
    // differences are exact when the cloud spans less than 2^30 record units
    bool ok = true;
    for (int k = 0; k < 2; k++)
    {
      double step = fabs(g.scale[k] * g.unit);
      ok = ok && step > 0 && (int64_t)c->grid.imax[k] - (int64_t)c->grid.imin[k] < ((int64_t)1 << 30) &&
           (g.tile_side + 4 * g.spacing) / step < (double)(1 << 30);
    }
    a.fast = ok ? 1 : 0;
  }
  a.sx = (const int32_t *)c->sx.p;
  a.sy = (const int32_t *)c->sy.p;
  a.sz = (const int32_t *)c->sz.p;
  a.xyzd = (const double *)c->xyzd.p;
  a.nd = c->nd;
  return a;
}

/* Puts the points of tiles above kFillMax points in store order (the order
 * OctStore::pointsIn returns), all such tiles in one radix sort. */
static int sortHugeTiles(wb_ctx *c, uint32_t nh, const uint32_t *tileStart)
{
  std::vector<uint32_t> list(nh), last(nh);
  std::vector<uint64_t> pre(nh + 1, 0);
  WB_CUDA(c, cudaMemcpyAsync(list.data(), c->tileHuge.p, nh * 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  const uint32_t *tileN = (const uint32_t *)c->tileN.p;
  for (uint32_t h = 0; h < nh; h++)
    WB_CUDA(c, cudaMemcpyAsync(&last[h], tileN + list[h], 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  for (uint32_t h = 0; h < nh; h++)
    pre[h + 1] = pre[h] + last[h];
  const uint64_t total = pre[nh];
  int rc;
  if ((rc = wb_ensure(c, c->hugePre, (nh + 1) * 8 + 64)) || (rc = wb_ensure(c, c->key0, total * 8 + 64)) ||
      (rc = wb_ensure(c, c->key1, total * 8 + 64)) || (rc = wb_ensure(c, c->idx0, total * 4 + 64)) ||
      (rc = wb_ensure(c, c->idx1, total * 4 + 64)))
    return rc;
  WB_CUDA(c, cudaMemcpyAsync(c->hugePre.p, pre.data(), (nh + 1) * 8, cudaMemcpyDefault, c->stream));
  uint64_t *keys = (uint64_t *)c->key0.p;
  uint32_t *vals = (uint32_t *)c->idx0.p;
  unsigned g = (unsigned)std::min<uint64_t>((total + 255) / 256 + 1, (uint64_t)c->sm_count * 16);
  { hugeKeysKernel<<<g, 256, 0, c->stream>>>(nh, (const uint32_t *)c->tileHuge.p, tileStart, (const uint64_t *)c->hugePre.p,
                                             (const uint32_t *)c->tilePts.p, keys, vals); ++c->launches; }
  int bits = 1;
  while ((1ull << bits) < nh)
    bits++;
  if ((rc = wb_radix_sort_pairs(c, keys, vals, (uint64_t *)c->key1.p, (uint32_t *)c->idx1.p, total, 0, 32 + bits)))
    return rc;
  { hugeBackKernel<<<g, 256, 0, c->stream>>>(nh, (const uint32_t *)c->tileHuge.p, tileStart, (const uint64_t *)c->hugePre.p,
                                             keys, (uint32_t *)c->tilePts.p); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  return 0;
}

/* Per tile, over its points (x, y from the tile centre, z as decoded): the
 * largest |r - r_ref| and |r_ref| of the fit residuals r = z - (a x + b y + c)
 * under the last scan's plane and r_ref under a given plane (NaN where
 * either plane is singular).  One warp per tile. */
__global__ void residualKernel(ScanArgs s, const TileRes *__restrict__ res, const double *__restrict__ ref,
                               double *__restrict__ maxDiff, double *__restrict__ maxRef)
{
  const int lane = threadIdx.x & 31;
  const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t k = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < s.t.T; k += warps)
  {
    double cx, cy;
    tileCenter(s.t, k, cx, cy);
    const double a = res[k].plane[0], b = res[k].plane[1], c = res[k].plane[2];
    const double ar = ref[3 * k], br = ref[3 * k + 1], cr = ref[3 * k + 2];
    double md = 0, mr = 0;
    const uint32_t base = s.tileStart[k], n = s.tileN[k];
    for (uint32_t t = lane; t < n; t += 32)
    {
      const uint32_t j = s.tilePts[base + t];
      const double x = dec(s.t, 0, s.t.sx[j]) - cx, y = dec(s.t, 1, s.t.sy[j]) - cy, z = dec(s.t, 2, s.t.sz[j]);
      const double r = z - (a * x + b * y + c), rr = z - (ar * x + br * y + cr);
      md = fmax(md, fabs(r - rr));
      mr = fmax(mr, fabs(rr));
    }
    for (int o = 16; o; o >>= 1)
    {
      md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
      mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
    }
    if (lane == 0)
    {
      const bool bad = !(a == a && b == b && c == c && ar == ar && br == br && cr == cr);
      maxDiff[k] = bad ? NAN : md;
      maxRef[k] = bad ? NAN : mr;
    }
  }
}

/* Sum of the tiles' room bounds in 64 bits. */
__global__ void boundTotal64(const uint32_t *bound, uint64_t T, unsigned long long *tot)
{
  unsigned long long s = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < T; i += (uint64_t)gridDim.x * blockDim.x)
    s += bound[i];
  for (int o = 16; o; o >>= 1)
    s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s)
    atomicAdd(tot, s);
}

int wb_scan_impl(wb_ctx *c, const wb_params *p)
{
  if (c->stage < 1)
    return wb_fail(c, WB_ESTATE, "wb_scan_tiles: build the octree first");
  if (!(p->tile_size > 0))
    return wb_fail(c, WB_EINVAL, "wb_scan_tiles: tile_size must be > 0");
  c->params = *p;
  WbGeom &g = c->g;
  wb_snake_size(g.tile_side, p->tile_size, &g.snake_idx, &g.spacing, &g.tile_lo, &g.tile_hi);
  int rc = uploadTiles(c);
  if (rc)
    return rc;
  uint64_t T = c->n_tiles, nd = c->nd;
  if ((rc = wb_ensure(c, c->tileN, T * 4 + 64)) || (rc = wb_ensure(c, c->tileStart, (T + 1) * 4 + 64)) ||
      (rc = wb_ensure(c, c->owner, nd * 4 + 64)) || (rc = wb_ensure(c, c->tileRes, T * sizeof(TileRes) + 64)) ||
      (rc = wb_ensure(c, c->tileH, T * 8 + 64)) || (rc = wb_ensure(c, c->small, 4096)))
    return rc;
  TileArgs a = tileArgs(c);
  GridDev gd;
  gd.x0 = c->grid.x0;
  gd.y0 = c->grid.y0;
  gd.cell = c->grid.cell;
  gd.nx = c->grid.nx;
  gd.ny = c->grid.ny;
  gd.ncell = c->grid.ncell;
  gd.cell2 = (const int4 *)c->cellRec.p;
  gd.gpt = (const int4 *)c->gpt.p;
  gd.leafId = (const uint32_t *)c->leafId.p;
  uint32_t *tileN = (uint32_t *)c->tileN.p, *tileStart = (uint32_t *)c->tileStart.p;
  int32_t *owner = (int32_t *)c->owner.p;
  unsigned blocks = (unsigned)((T + kTileWarps - 1) / kTileWarps);
  // room per tile (tileNg holds the bounds until the fill reuses it as its list)
  if ((rc = wb_ensure(c, c->tileNg, T * 4 + 64)))
    return rc;
  uint32_t *bound = (uint32_t *)c->tileNg.p;
  if ((rc = wb_ensure(c, c->tileFrm, T * sizeof(TileFrame) + 64)))
    return rc;
  TileFrame *frames = (TileFrame *)c->tileFrm.p;
  { gridBound<<<(unsigned)std::min<uint64_t>((T + 127) / 128, (uint64_t)c->sm_count * 32), 128, 0, c->stream>>>(
        a, gd, bound, frames); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  uint32_t *dTot = (uint32_t *)((char *)c->small.p + 64);
  // Cylinders overlap, so the rooms add up to more than the points; their sum
  // is taken in 64 bits first, because the list offsets below are 32-bit.
  unsigned long long *dTot64 = (unsigned long long *)((char *)c->small.p + 768);
  WB_CUDA(c, cudaMemsetAsync(dTot64, 0, 8, c->stream));
  { boundTotal64<<<(unsigned)std::min<uint64_t>((T + 255) / 256, (uint64_t)c->sm_count * 8), 256, 0, c->stream>>>(
        bound, T, dTot64); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  unsigned long long room64 = 0;
  WB_CUDA(c, cudaMemcpyAsync(&room64, dTot64, 8, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (room64 > 0xfffffff0ull)
    return wb_fail(c, WB_EINVAL, "wb_scan_tiles: the tiles' point lists would hold " + std::to_string(room64) +
                                     " entries, above the 2^32 that their 32-bit offsets address");
  if ((rc = wb_exclusive_scan_u32(c, bound, tileStart, T, dTot)))
    return rc;
  WB_CUDA(c, cudaMemcpyAsync(tileStart + T, dTot, 4, cudaMemcpyDefault, c->stream));
  uint32_t room = (uint32_t)room64;
  if ((rc = wb_ensure(c, c->tilePts, (uint64_t)room * 4 + 64)))
    return rc;
  { fillOwner<<<(unsigned)std::min<uint64_t>((nd + 255) / 256 + 1, (uint64_t)c->sm_count * 16), 256, 0, c->stream>>>(owner, nd); ++c->launches; }
  int *dOvf = (int *)((char *)c->small.p + 384);
  uint32_t *dBig = (uint32_t *)((char *)c->small.p + 392);
  // huge-tile count and big-tile count (bytes 384..395 of the scratch block)
  WB_CUDA(c, cudaMemsetAsync(dOvf, 0, 16, c->stream));
  { gridFillWarp<<<blocks, 32 * kTileWarps, 0, c->stream>>>(a, gd, tileStart, tileN, (uint32_t *)c->tilePts.p, owner,
                                                           (uint32_t *)c->tileNg.p, dBig, frames); ++c->launches; }
  if ((rc = wb_ensure(c, c->tileHuge, T * 4 + 64)))
    return rc;
  { gridFill<<<(unsigned)c->sm_count, kFillThreads, 0, c->stream>>>(a, gd, tileStart, tileN, (uint32_t *)c->tilePts.p,
                                                                   owner, dOvf, (const uint32_t *)c->tileNg.p, dBig,
                                                                   (uint32_t *)c->tileHuge.p, frames); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  int nHuge = 0;
  WB_CUDA(c, cudaMemcpyAsync(&nHuge, dOvf, 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (nHuge && (rc = sortHugeTiles(c, (uint32_t)nHuge, tileStart)))
    return rc;
  wb_mark(c, "tile_gather");
  ScanArgs s;
  s.t = a;
  s.tileStart = tileStart;
  s.tileN = tileN;
  s.tilePts = (const uint32_t *)c->tilePts.p;
  s.minH = p->min_hyp_size;
  TileRes *res = (TileRes *)c->tileRes.p;
  // one work slot per tile (64 B, 80 B in the precision mode); the centres
  // come from the tile frames
  if ((rc = wb_ensure(c, c->scanTot, T * sizeof(ScanWork32) + 64)))
    return rc;
  const unsigned sb = (unsigned)((T + kScanWarps - 1) / kScanWarps);
  const unsigned tb = (unsigned)std::min<uint64_t>((T + 127) / 128, (uint64_t)c->sm_count * 32);
  if (c->precision == WB_PRECISION_FP32 && a.fast)
  {
    ScanWork32 *work = (ScanWork32 *)c->scanTot.p;
    { scan32Sums<<<sb, 32 * kScanWarps, 0, c->stream>>>(s, work); ++c->launches; }
    { scan32Solve<<<tb, 128, 0, c->stream>>>(a, tileN, frames, work, res); ++c->launches; }
    { scan32Shape<<<sb, 32 * kScanWarps, 0, c->stream>>>(s, frames, work); ++c->launches; }
    { scanFinish<<<tb, 128, 0, c->stream>>>(T, tileN, work, a.rad, p->min_hyp_size, res); ++c->launches; }
  }
  else
  {
    ScanWork *work = (ScanWork *)c->scanTot.p;
    { scanSums<<<sb, 32 * kScanWarps, 0, c->stream>>>(s, frames, work); ++c->launches; }
    { scanSolve<<<tb, 128, 0, c->stream>>>(T, tileN, work, res); ++c->launches; }
    { scanShape<<<sb, 32 * kScanWarps, 0, c->stream>>>(s, frames, work); ++c->launches; }
    { scanFinish<<<tb, 128, 0, c->stream>>>(T, tileN, work, a.rad, p->min_hyp_size, res); ++c->launches; }
  }
  WB_CUDA(c, cudaGetLastError());
  wb_mark(c, "scan");
  unsigned pb = (unsigned)std::min<uint64_t>((T + 255) / 256, (uint64_t)c->sm_count * 16);
  { postscanKernel<<<pb, 256, 0, c->stream>>>(T, a.ex, a.ey, (const int32_t *)c->tileLookup.p, c->lookupX0, c->lookupY0,
                                            c->lookupW, c->lookupH, g.spacing, res, (double *)c->tileH.p); ++c->launches; }
  { applyH<<<pb, 256, 0, c->stream>>>(T, (const double *)c->tileH.p, res); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  wb_mark(c, "postscan");
  c->stage = 2;
  return 0;
}

int wb_tile_residuals(wb_ctx *c, const double *abc_ref, double *max_diff, double *max_ref)
{
  if (!c || !abc_ref || !max_diff || !max_ref)
    return WB_EINVAL;
  if (c->stage < 2)
    return wb_fail(c, WB_ESTATE, "wb_tile_residuals: scan the tiles first");
  WbDeviceGuard deviceGuard(c->device);
  const uint64_t T = c->n_tiles;
  if (T == 0)
    return 0;
  WbScratch ref(c), out(c);
  int rc;
  if ((rc = wb_ensure(c, ref.b, T * 24 + 64)) || (rc = wb_ensure(c, out.b, T * 16 + 64)))
    return rc;
  WB_CUDA(c, cudaMemcpyAsync(ref.b.p, abc_ref, T * 24, cudaMemcpyDefault, c->stream));
  ScanArgs s;
  s.t = tileArgs(c);
  s.tileStart = (const uint32_t *)c->tileStart.p;
  s.tileN = (const uint32_t *)c->tileN.p;
  s.tilePts = (const uint32_t *)c->tilePts.p;
  s.minH = c->params.min_hyp_size;
  double *md = (double *)out.b.p, *mr = md + T;
  { residualKernel<<<(unsigned)std::min<uint64_t>((T * 32 + 255) / 256, (uint64_t)c->sm_count * 32), 256, 0,
                     c->stream>>>(s, (const TileRes *)c->tileRes.p, (const double *)ref.b.p, md, mr); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  WB_CUDA(c, cudaMemcpyAsync(max_diff, md, T * 8, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaMemcpyAsync(max_ref, mr, T * 8, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  return 0;
}

/* classifyCylinder on the GPU (classify.cpp:96-173).
 *
 * The reference classifies point p by growing a std::set of integer
 * directions dir(p,q) to the points q inside the downward hyperboloid
 * Hyperboloid(p - (0,0,thickness), tile.hyperboloidSize, maxSlope), stopping
 * as soon as no circular gap between successive directions reaches 144
 * degrees (surround, classify.cpp:67-94).  Adding directions can only shrink
 * gaps, and the pruning surround() does never opens one, so the label is a
 * function of the neighbour set alone: 1 (not ground) if it surrounds p, else 2.
 * The neighbour set is what OctStore::pointsIn returns for the hyperboloid.
 *
 * Two kernels walk the same neighbourhood.  The column-group kernel
 * (classifyGroup, the fast pass) gives one warp to up to 32 points of one
 * grid column and shares the walk between them; the one-point kernel
 * (classifyPoint) gives one warp to one point and serves the points a group
 * hands over, and the exact pass.  Both walk rings of grid columns outward
 * from the point, so directions from every side arrive early, and stop as soon
 * as the directions seen surround the point.  Per column they first check
 * whether the column's lowest point could be inside the hyperboloid at the
 * column's nearest distance.  Each candidate is tested in FP32 in a frame centred on p
 * (integer record differences times the scale); the few whose FP32 value lies
 * within 1e-5 of the boundary, and points outside the octree root cube (which
 * the reference treats through their leaf's cube), are tested exactly in
 * FP64 as the reference computes it.  Directions are FP32 arctangents
 * (wb_dir_units_f32, error below 1000 units) in the reference's integer angle
 * unit; bins (64 in the one-point kernel, 8 per lane in the group kernel) keep
 * their extremes, and the largest circular gap follows from them.  With the direction error bounded by kMargin units, a
 * gap estimate below 144 degrees - 2*kMargin proves "surrounded" and one
 * above 144 degrees + 2*kMargin proves the opposite;
 * anything between is re-run by the exact kernel with the reference's own
 * integer atan2i (angle.cpp:117-155) and exact bins.
 *
 * A point is classified with the hyperboloid size of its owner tile, the last
 * tile in flowsnake order whose cylinder contains it, because that tile's
 * classification is the one the reference keeps.
 */
#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#include "wb_internal.h"
#include "wb_device.cuh"
#include "angle_tables.h"

/* Work counters of the classify kernel, compiled in only with
 * -DWB_CLASSIFY_STATS (an instrumented build for tuning): per label,
 * 0 points, 1 near columns tested, 2 super-cells tested, 3 far columns
 * tested, 4 candidates read, 5 candidates inside, 6 surround tests,
 * 7 columns scanned; SM clock cycles 8 near field, 9 far field, 10 final
 * gap, 11 whole point, 12 inside column scans, 13 inside surround tests.
 * Row 0 is the column-group kernel: 0 groups, 1 columns read, 2 candidates
 * kept, 3 kept x undecided lanes, 4 active lanes, 5 lanes handed over,
 * 6 cycles, 7 super-cell rings, 8 lanes ending ground; 9-11 cycles, count
 * and kept candidates of the groups that kept more than 1000; cycles 12 in
 * column reads, 13 forming the envelope again, 14 candidate tests, 15
 * surround tests. */
#ifdef WB_CLASSIFY_STATS
__device__ unsigned long long gClassifyStats[3][16];
extern "C" int wb_classify_stats(unsigned long long *out, int reset)
{
  if (cudaMemcpyFromSymbol(out, gClassifyStats, sizeof(gClassifyStats)) != cudaSuccess)
    return -3;
  if (reset)
  {
    unsigned long long z[48] = {0};
    cudaMemcpyToSymbol(gClassifyStats, z, sizeof(z));
  }
  return 0;
}
#define WB_STAT(var, v) (var) += (v)
#else
#define WB_STAT(var, v) ((void)0)
#endif

namespace
{
constexpr int kBins = 64;
constexpr uint32_t kStray = 0x80000000u;
/* bound on |FP32 direction - atan2i| in angle units (2^31 per turn); the
 * FP32 direction (wb_dir_units_f32) stays below 1000 units (tested against
 * atan2i on random and edge-case differences), so this is twice that. */
constexpr uint32_t kMargin = 2048;

/* Radians per unit of the reference's integer angle (2^31 per turn). */
constexpr float kUnitRad = 2.925836158534319e-09f;
/* How far an arc's rays are moved outward: far above the FP32 direction's
 * error bound (kMargin units, 6e-6 rad), the arc endpoints' float rounding
 * (128 units) and the box test's rounding. */
constexpr float kArcPad = 4e-5f;

/* Per-point values the warp kernel needs, formed once per point by a
 * thread-per-point kernel: double arithmetic costs 16 cycles per warp
 * instruction on this GPU, so it is kept out of the 32-lane warp kernel. */
struct PtSetup
{
  float czp, por2f;   /* cz - pz and por^2 (FP32)                         */
  int32_t ci, cj;     /* column of the point (may lie outside the grid)   */
  int32_t kmax, smax; /* rings of columns / super-cells the reach needs   */
};

struct ClsArgs
{
  uint64_t nd;
  double off[3], scale[3], unit;
  double slope, thickness;
  const uint64_t *leafKey;
  const uint8_t *leafLev;
  const uint32_t *leafId;
  double rootLo[3], rootSide;
  const int32_t *sx, *sy, *sz;
  const double *xyzd;   /* decoded x, y, z planes of nd doubles */
  const int32_t *owner;
  const TileRes *tiles;
  const double *tanT, *sinT, *cosT;
  uint8_t *label;
  /* grid */
  double gx0, gy0, cell;
  double invSlope2;          /* 1/slope^2, for the reach bound */
  float invCellF, invSuperF; /* 1/cell, 1/(WB_SUPER cell) in FP32, for the ring counts */
  const int2 *colOf;         /* column of each stored point, from the grid build */
  int nx, ny;
  uint64_t ncell;
  const int4 *col;     /* two int4 per column: {x0, y0, x1, y1}, {zmin, begin, end, flags} */
  const int4 *gpt;     /* int4 {X, Y, Z, position | stray bit} per point, column order */
  const uint2 *groups; /* column groups: {column, first point} */
  int snx, sny;
  const int4 *super;   /* super-cell records, the column layout */
  double zmin;
  int exactInts;   /* decode strictly increasing and 32-bit record differences exact */
  int fp32Only;    /* precision mode: FP32 decisions stand, no exact re-run */
  float fsx, fsy, fsz, fs2;   /* metres per record unit and slope^2, FP32 */
  PtSetup *setup;
  /* ambiguous points for the exact pass */
  uint32_t *ambList;
  uint32_t *ambCount;
  /* points a column group handed to the one-point kernel */
  uint32_t *deferList;
  uint32_t *deferCount;
  const uint32_t *work;   /* exact pass: store positions to classify */
  uint32_t nwork;
  /* finishing (fused launch): records, their store positions and class bytes */
  uint64_t n, nTiles;
  const uint32_t *storeOf;
  uint8_t *cls;
  /* decision margins (wb_classify_ex): per store position, and per record */
  float *margin, *marginOut;
};

/* Decision margin of a point in degrees: the largest gap between its
 * neighbours' directions minus 144 degrees (negative: surrounded, not
 * ground); with fewer than two directions there is no gap to speak of and
 * the point is ground by 216 degrees. */
__device__ __forceinline__ float marginDeg(uint32_t gap, bool twoDirs)
{
  return twoDirs ? (float)((double)gap - (double)WB_DEG144) * (float)(360.0 / 2147483648.0) : 216.f;
}

__device__ __forceinline__ double decA(const ClsArgs &a, int ax, int32_t q)
{
  return wb_decode(q, a.off[ax], a.scale[ax], a.unit);
}

struct Hyp
{
  int32_t qx, qy, qz;           /* the point, record integers                          */
  float sx, sy, sz;             /* metres per record unit                              */
  float czp, s2, por2f;         /* cz - pz, slope^2, por^2 in FP32                     */
  uint32_t j;                   /* store position of the point                         */
};

/* The exact Hyperboloid of point j: centre and polar radius squared, as
 * shape.cpp:119-125 forms them from p - (0,0,thickness). */
struct HypExact
{
  double cx, cy, cz, por2, px, py;
};

__device__ __noinline__ HypExact exactHyp(const ClsArgs &a, uint32_t j)
{
  HypExact e;
  double hs = a.tiles[a.owner[j]].h;
  e.px = decA(a, 0, a.sx[j]);
  e.py = decA(a, 1, a.sy[j]);
  double pz = decA(a, 2, a.sz[j]);
  double por = hs * (a.slope * a.slope);
  e.por2 = por * por;
  e.cx = e.px + 0;
  e.cy = e.py + 0;
  e.cz = (pz - a.thickness) + por;
  return e;
}

/* OctStore::pointsIn membership of one candidate, exactly: Hyperboloid::in on
 * the decoded doubles; for a point outside the root cube, its leaf cube must
 * meet the hyperboloid (Octree::findBlocks) and then either all eight corners
 * are inside (the whole block is taken) or the point itself is. */
__device__ __noinline__ bool memberExact(const ClsArgs &a, const HypExact &h, uint32_t gp, int32_t qx, int32_t qy,
                                         int32_t qz)
{
  double x = decA(a, 0, qx), y = decA(a, 1, qy), z = decA(a, 2, qz);
  bool in = wb_hyp_in(h.cx, h.cy, h.cz, h.por2, a.slope, x, y, z);
  if (!(gp & kStray))
    return in;
  uint32_t l = a.leafId[gp & ~kStray];
  double lx, ly, lz, ls;
  wb_leaf_cube(a.leafKey[l], a.leafLev[l], a.rootLo, a.rootSide, lx, ly, lz, ls);
  if (!wb_hyp_in(h.cx, h.cy, h.cz, h.por2, a.slope, wb_clamp_toward(h.cx, lx, ls), wb_clamp_toward(h.cy, ly, ls),
                 lz - ls / 2))
    return false;
  bool all = true;
  for (int n = 0; n < 8 && all; n++)
    all = wb_hyp_in(h.cx, h.cy, h.cz, h.por2, a.slope, (n & 1) ? lx + ls / 2 : lx - ls / 2,
                    (n & 2) ? ly + ls / 2 : ly - ls / 2, (n & 4) ? lz + ls / 2 : lz - ls / 2);
  return all || in;
}

/* Can any point of a box (integer bounds, 6 planes of N entries) be inside?
 * FP32 with generous slack.  Record differences are exact in 32 bits: the
 * host checks that the cloud's integer extent fits. */
__device__ __forceinline__ bool boxMeets(const Hyp &h, const int4 &b, int32_t zmin)
{
  if (b.x == INT32_MAX)
    return false;   // empty block
  // the bound takes the box's low record integers as its low coordinates:
  // only for a decode that increases with the record integer
  if (!(h.sx > 0.f && h.sy > 0.f && h.sz > 0.f))
    return true;
  float xl = (float)(b.x - h.qx) * h.sx, xh = (float)(b.z - h.qx) * h.sx;
  float yl = (float)(b.y - h.qy) * h.sy, yh = (float)(b.w - h.qy) * h.sy;
  float zd = (float)(h.qz - zmin) * h.sz + h.czp;
  float dx = xl > 0 ? xl : (xh < 0 ? -xh : 0.f);
  float dy = yl > 0 ? yl : (yh < 0 ? -yh : 0.f);
  float r2 = h.s2 * (dx * dx + dy * dy);
  float mag = zd * zd + r2 + h.por2f;
  if (zd < -1e-4f * (fabsf(zd) + 1e-3f))
    return false;
  return zd * zd - r2 - h.por2f >= -(1e-4f * mag + 1e-9f);
}

/* Column offset of ring cell m (0 <= m < 8k) at Chebyshev distance k. */
__device__ __forceinline__ void ringCell(int k, int m, int &di, int &dj)
{
  if (k == 0)
  {
    di = dj = 0;
    return;
  }
  int side = m / (2 * k), o = m % (2 * k);
  if (side == 0)
  {
    di = -k + o;
    dj = -k;
  }
  else if (side == 1)
  {
    di = k;
    dj = -k + o;
  }
  else if (side == 2)
  {
    di = k - o;
    dj = k;
  }
  else
  {
    di = -k;
    dj = k - o;
  }
}

/* Largest circular gap between occupied bins' extremes; lanes hold 2 bins. */
__device__ __forceinline__ uint32_t largestGap(const uint32_t *bmin, const uint32_t *bmax, int lane, int &nocc)
{
  uint32_t mn0 = bmin[lane], mn1 = bmin[lane + 32];
  uint32_t mx0 = bmax[lane], mx1 = bmax[lane + 32];
  unsigned lo = __ballot_sync(0xffffffffu, mn0 != 0xffffffffu);
  unsigned hi = __ballot_sync(0xffffffffu, mn1 != 0xffffffffu);
  uint64_t occ = ((uint64_t)hi << 32) | lo;
  nocc = __popcll(occ);
  uint32_t worst = 0;
  if (nocc >= 2)
  {
    for (int half = 0; half < 2; half++)
    {
      int b = lane + 32 * half;
      if ((occ >> b) & 1)
      {
        uint64_t rot = (b == 63) ? 0 : (occ >> (b + 1));
        int nb = rot ? b + 1 + __ffsll((long long)rot) - 1 : __ffsll((long long)occ) - 1;
        uint32_t gap = (bmin[nb] - (half ? mx1 : mx0)) & 0x7fffffffu;
        worst = max(worst, gap);
      }
    }
    for (int o = 16; o; o >>= 1)
      worst = max(worst, __shfl_xor_sync(0xffffffffu, worst, o));
  }
  return worst;
}

/* largestGap, plus the gaps at or above thr: how many there are and, for the
 * last one found, where it starts (u0, a bin's largest direction) and how
 * wide it is; every lane receives the same values. */
__device__ __forceinline__ uint32_t largestGapArc(const uint32_t *bmin, const uint32_t *bmax, int lane, uint32_t thr,
                                                  int &nocc, int &nbig, uint32_t &u0, uint32_t &w)
{
  uint32_t mn0 = bmin[lane], mn1 = bmin[lane + 32];
  uint32_t mx0 = bmax[lane], mx1 = bmax[lane + 32];
  unsigned lo = __ballot_sync(0xffffffffu, mn0 != 0xffffffffu);
  unsigned hi = __ballot_sync(0xffffffffu, mn1 != 0xffffffffu);
  uint64_t occ = ((uint64_t)hi << 32) | lo;
  nocc = __popcll(occ);
  nbig = 0;
  u0 = w = 0;
  uint32_t worst = 0, myU0 = 0, myW = 0;
  bool big = false;
  if (nocc >= 2)
  {
    for (int half = 0; half < 2; half++)
    {
      int b = lane + 32 * half;
      if ((occ >> b) & 1)
      {
        uint64_t rot = (b == 63) ? 0 : (occ >> (b + 1));
        int nb = rot ? b + 1 + __ffsll((long long)rot) - 1 : __ffsll((long long)occ) - 1;
        const uint32_t start = half ? mx1 : mx0;
        uint32_t gap = (bmin[nb] - start) & 0x7fffffffu;
        worst = max(worst, gap);
        if (gap >= thr)
        {
          nbig += 1;
          big = true;
          myU0 = start;
          myW = gap;
        }
      }
    }
    for (int o = 16; o; o >>= 1)
    {
      worst = max(worst, __shfl_xor_sync(0xffffffffu, worst, o));
      nbig += __shfl_xor_sync(0xffffffffu, nbig, o);
    }
    const unsigned bl = __ballot_sync(0xffffffffu, big);
    if (bl)
    {
      const int src = 31 - __clz(bl);
      u0 = __shfl_sync(0xffffffffu, myU0, src);
      w = __shfl_sync(0xffffffffu, myW, src);
    }
  }
  return worst;
}

/* The double-precision set-up of point j's query, one thread per point. */
__device__ __forceinline__ void setupPoint(const ClsArgs &a, uint64_t j)
{
  int32_t k = a.owner[j];
  if (k < 0)
    return;
  double hs = a.tiles[k].h;
  const double pz = a.xyzd[2 * a.nd + j];
  double por = hs * (a.slope * a.slope);
  double por2 = por * por;
  double cz = (pz - a.thickness) + por;
  PtSetup s;
  s.czp = (float)(cz - pz);
  s.por2f = (float)por2;
  // horizontal reach of the hyperboloid at the lowest point of the cloud
  double zdMax = cz - a.zmin;
  // The ring counts only bound the search (columns beyond the reach hold no
  // member), so they are formed in FP32 with a 1e-5 margin, far above the
  // 1e-7 rounding of the FP32 root and products.
  const float r2f = (float)((zdMax * zdMax - por2) * a.invSlope2);
  const float reach = r2f > 0 ? sqrtf(r2f) * (1 + 1e-5f) + 1e-5f : 0.f;
  const int2 col = a.colOf[j];
  s.ci = col.x;
  s.cj = col.y;
  s.kmax = (int32_t)fminf(ceilf(reach * a.invCellF) + 1, 1e9f);
  s.smax = (int32_t)fminf(ceilf(reach * a.invSuperF) + 1, 1e9f);
  a.setup[j] = s;
}

/* Classifies store position j with one warp; bminW/bmaxW are the warp's
 * 64-bin direction extremes in shared memory. */
template <bool EXACT>
__device__ __forceinline__ void classifyPoint(const ClsArgs &a, uint64_t j, int lane, uint32_t *bminW,
                                              uint32_t *bmaxW)
{
  int32_t k = a.owner[j];
  if (k < 0)
  {
    if (lane == 0)
    {
      a.label[j] = 0;
      if (a.margin)
        a.margin[j] = __int_as_float(0x7fc00000);
    }
    return;
  }
  Hyp h;
  h.qx = a.sx[j];
  h.qy = a.sy[j];
  h.qz = a.sz[j];
  h.j = (uint32_t)j;
  h.sx = a.fsx;
  h.sy = a.fsy;
  h.sz = a.fsz;
  h.s2 = a.fs2;
  const PtSetup ps = a.setup[j];
  h.czp = ps.czp;
  h.por2f = ps.por2f;
  for (int b = lane; b < kBins; b += 32)
  {
    bminW[b] = 0xffffffffu;
    bmaxW[b] = 0;
  }
  __syncwarp();
  const int ci = ps.ci, cj = ps.cj, kmax = ps.kmax;
  HypExact hx;
  if (EXACT)
    hx = exactHyp(a, (uint32_t)j);
  bool surrounded = false, ambiguous = false;
  // FP32 membership (exact: its band goes to FP64) and height bounds wherever
  // 32-bit record differences are exact; FP32 directions only in the fast pass
  const bool fp32Member = a.exactInts;
  const bool fast = !EXACT && a.exactInts;
  // Directions are kept as exact per-bin extremes in shared memory plus a
  // 64-bit occupancy mask in registers (uniform across the warp).
  uint32_t occLo = 0, occHi = 0;
  uint32_t gapNow = 0;   // the largest gap at the last surround test that formed it
  bool gapValid = false;
  // The point's arc (see setArc): directions outside the one gap that can
  // still decide the point change nothing, so boxes outside it are skipped.
  int amode = 0;
  float e0x = 0.f, e0y = 0.f, e1x = 0.f, e1y = 0.f;
  auto arcWants = [&](const int4 &mine, int src) -> bool {
    if (amode == 0)
      return true;
    int4 b;
    b.x = __shfl_sync(0xffffffffu, mine.x, src);
    b.y = __shfl_sync(0xffffffffu, mine.y, src);
    b.z = __shfl_sync(0xffffffffu, mine.z, src);
    b.w = __shfl_sync(0xffffffffu, mine.w, src);
    const float x0 = (float)(b.x - h.qx) * h.sx, x1 = (float)(b.z - h.qx) * h.sx;
    const float y0 = (float)(b.y - h.qy) * h.sy, y1 = (float)(b.w - h.qy) * h.sy;
    if (amode == 1)
    {
      const float A = fmaxf(e0x * y0, e0x * y1) + fmaxf(-e0y * x0, -e0y * x1);
      const float B = fmaxf(e1y * x0, e1y * x1) + fmaxf(-e1x * y0, -e1x * y1);
      const float bx = e0x + e1x, by = e0y + e1y;
      const float D = fmaxf(bx * x0, bx * x1) + fmaxf(by * y0, by * y1);
      return A >= 0.f && B >= 0.f && D >= 0.f;
    }
    const float A = fminf(e1x * y0, e1x * y1) + fminf(-e1y * x0, -e1y * x1);
    const float B = fminf(e0y * x0, e0y * x1) + fminf(-e0x * y0, -e0x * y1);
    return !(A > 0.f && B > 0.f);
  };
  unsigned long long stat[16] = {0};
#ifdef WB_CLASSIFY_STATS
  const long long tStart = clock64();
#endif
  (void)stat;
  // Points of a column are sorted by height.  None above pz + (czp -
  // sqrt(por^2 + s^2 d^2)) / sz, d the column's nearest distance, can be
  // inside: colZlim gives that bound (with slack) in record units relative to
  // the point.  Columns holding points outside the root cube in x or y get no
  // bound (their blocks' cubes decide for them).
  auto colZlim = [&](const int4 &box, const int4 &r1) -> int32_t {
    if (!fp32Member || r1.w || !(h.sz > 0))
      return INT32_MAX;
    float xl = (float)(box.x - h.qx) * h.sx, xh = (float)(box.z - h.qx) * h.sx;
    float yl = (float)(box.y - h.qy) * h.sy, yh = (float)(box.w - h.qy) * h.sy;
    float dx = xl > 0 ? xl : (xh < 0 ? -xh : 0.f);
    float dy = yl > 0 ? yl : (yh < 0 ? -yh : 0.f);
    float need = sqrtf(h.por2f + h.s2 * (dx * dx + dy * dy));
    float dz = (h.czp - need + 1e-4f * (fabsf(h.czp) + need) + 1e-6f) / h.sz + 2.f;
    return dz > 2.1e9f ? INT32_MAX : (dz < -2.1e9f ? INT32_MIN : (int32_t)floorf(dz));
  };
  // Whether candidate pt lies inside the hyperboloid, and its direction u.
  auto testPoint = [&](const int4 &pt, uint32_t &u) -> bool {
    bool in = false;
    const int32_t qx = pt.x, qy = pt.y, qz = pt.z;
    const uint32_t gp = (uint32_t)pt.w;
    if (fp32Member)
    {
      int32_t dxi = qx - h.qx, dyi = qy - h.qy;
      // dist(p,q) == 0 gives no direction (classify.cpp:142,153)
      if (dxi != 0 || dyi != 0)
      {
        float dx = (float)dxi * h.sx, dy = (float)dyi * h.sy;
        if (gp & kStray)
          in = memberExact(a, exactHyp(a, h.j), gp, qx, qy, qz);
        else
        {
          float dzm = (float)(h.qz - qz) * h.sz;
          float zd = dzm + h.czp;
          float r2 = h.s2 * (dx * dx + dy * dy);
          float f = zd * zd - r2 - h.por2f;
          float tol = 1e-5f * (zd * zd + r2 + h.por2f) + 1e-12f;
          float ztol = 1e-5f * (fabsf(dzm) + fabsf(h.czp)) + 1e-12f;
          if (zd > ztol && f > tol)
            in = true;
          else if (zd < -ztol || f < -tol)
            in = false;
          else if (a.fp32Only)
            in = zd > 0 && f > 0;
          else
            in = memberExact(a, exactHyp(a, h.j), gp, qx, qy, qz);
        }
        if (in && fast)
          u = (uint32_t)__float2int_rn(wb_dir_units_f32(dy, dx)) & 0x7fffffffu;
        else if (in)
        {
          // the exact pass: the reference's integer direction of the decoded points
          double x = decA(a, 0, qx), y = decA(a, 1, qy);
          u = (uint32_t)wb_atan2i(y - hx.py, x - hx.px, a.tanT, a.sinT, a.cosT, WB_ATAN_SCALE_HI,
                                  WB_ATAN_SCALE_LO) & 0x7fffffffu;
        }
      }
    }
    else
    {
      double x = decA(a, 0, qx), y = decA(a, 1, qy);
      if (wb_hypot(hx.px - x, hx.py - y) != 0 && memberExact(a, hx, gp, qx, qy, qz))
      {
        in = true;
        int d = wb_atan2i(y - hx.py, x - hx.px, a.tanT, a.sinT, a.cosT, WB_ATAN_SCALE_HI, WB_ATAN_SCALE_LO);
        u = (uint32_t)d & 0x7fffffffu;
      }
    }
    return in;
  };
  // Merges the directions of a chunk's inside lanes into the bins; returns
  // whether any lane was inside.
  auto merge = [&](bool in, uint32_t u) -> bool {
    if (!__any_sync(0xffffffffu, in))
      return false;
    // Directions of nearby points usually share one bin: then one lane
    // merges the warp's extremes; otherwise each lane does.
    uint32_t bin = u >> 25;
    uint32_t lo = __reduce_min_sync(0xffffffffu, in ? u : 0xffffffffu);
    uint32_t hi = __reduce_max_sync(0xffffffffu, in ? u : 0u);
    if ((lo >> 25) == (hi >> 25))
    {
      if (lane == 0)
      {
        atomicMin(&bminW[lo >> 25], lo);
        atomicMax(&bmaxW[lo >> 25], hi);
      }
      if ((lo >> 25) < 32)
        occLo |= 1u << (lo >> 25);
      else
        occHi |= 1u << ((lo >> 25) - 32);
    }
    else
    {
      if (in)
      {
        atomicMin(&bminW[bin], u);
        atomicMax(&bmaxW[bin], u);
      }
      occLo |= __reduce_or_sync(0xffffffffu, in && bin < 32 ? 1u << bin : 0u);
      occHi |= __reduce_or_sync(0xffffffffu, in && bin >= 32 ? 1u << (bin - 32) : 0u);
    }
    WB_STAT(stat[5], __popc(__ballot_sync(0xffffffffu, in)));
    return true;
  };
  // Adds the directions of column cc's inside points; returns whether any was.
  auto column = [&](uint64_t cc) -> bool {
    WB_STAT(stat[7], 1);
#ifdef WB_CLASSIFY_STATS
    const long long tc = clock64();
#endif
    bool got = false;
    const int4 box = a.col[2 * cc], r1 = a.col[2 * cc + 1];
    const uint32_t e = (uint32_t)r1.z;
    const int32_t zlim = colZlim(box, r1);
    for (uint32_t t0 = (uint32_t)r1.y; t0 < e; t0 += 32)
    {
      uint32_t t = t0 + lane;
      bool low = false;
      int4 pt = make_int4(0, 0, 0, 0);
      if (t < e)
      {
        pt = a.gpt[t];
        low = zlim == INT32_MAX || pt.z - h.qz <= zlim;
      }
      // the scan stops at the first chunk wholly past the height bound
      if (!__any_sync(0xffffffffu, low))
        break;
      WB_STAT(stat[4], __popc(__ballot_sync(0xffffffffu, low)));
      uint32_t u = 0;
      bool in = low && testPoint(pt, u);
      got |= merge(in, u);
    }
    WB_STAT(stat[12], clock64() - tc);
    return got;
  };
  // Surround test from the bin extremes; it also gives the arc.  The fast
  // pass decides two margins away from 144 degrees, exact directions (the
  // exact pass, clouds without exact 32-bit differences) and the precision
  // mode at 144 degrees.  The arc is as sound with exact directions: only a
  // direction inside the one gap at or above the threshold can change the
  // label or the largest gap.
  auto decideBody = [&]() {
    WB_STAT(stat[6], 1);
    uint64_t occ = ((uint64_t)occHi << 32) | occLo;
    if (__popcll(occ) < 2)
      return;
    {
      __syncwarp();
      int nocc, nbig;
      uint32_t u0, w;
      const bool at144 = !fast || a.fp32Only;
      const uint32_t thr = at144 ? (uint32_t)WB_DEG144 : (uint32_t)WB_DEG144 - 2 * kMargin;
      uint32_t gap = largestGapArc(bminW, bmaxW, lane, thr, nocc, nbig, u0, w);
      gapNow = gap;
      gapValid = nocc >= 2;
      if (nocc >= 2)
        surrounded = at144 ? gap < (uint32_t)WB_DEG144 : gap + 2 * kMargin < (uint32_t)WB_DEG144;
      amode = 0;
      if (!surrounded && nbig == 1)
      {
        const float a0 = (float)u0 * kUnitRad - kArcPad;
        const float W = (float)w * kUnitRad + 2.f * kArcPad;
        if (W < 6.2f)
        {
          float s0, c0, s1, c1;
          const float a1 = a0 + W;
          __sincosf(a0 > 3.14159265f ? a0 - 6.28318531f : a0, &s0, &c0);
          __sincosf(a1 > 3.14159265f ? (a1 > 9.42477796f ? a1 - 12.56637061f : a1 - 6.28318531f) : a1, &s1, &c1);
          e0x = c0;
          e0y = s0;
          e1x = c1;
          e1y = s1;
          amode = W < 3.14159f ? 1 : 2;
        }
      }
    }
  };
  auto decide = [&]() {
#ifdef WB_CLASSIFY_STATS
    const long long td = clock64();
#endif
    decideBody();
    WB_STAT(stat[13], clock64() - td);
  };
  // Near field: rings of single columns around the point's column, each ring
  // visited in an order that alternates sides (stride 4k-1 over its 8k
  // columns), with the surround test after every column.  One ring (nine
  // columns) measured fastest; the super-cell rings take over beyond it.
  const int kNear = 1;
  for (int ring = 0; ring <= kNear && ring <= kmax && !surrounded; ring++)
  {
    if (ci + ring < 0 || ci - ring >= a.nx || cj + ring < 0 || cj - ring >= a.ny)
      continue;
    int ncells = ring == 0 ? 1 : 8 * ring;
    int stride = ring == 0 ? 1 : 4 * ring - 1;
    WB_STAT(stat[1], ncells);
    for (int m0 = 0; m0 < ncells && !surrounded; m0 += 32)
    {
      int m = m0 + lane;
      uint64_t c = 0;
      bool ok = false;
      int4 cb = make_int4(0, 0, 0, 0);
      if (m < ncells)
      {
        int di, dj;
        ringCell(ring, (m * stride) % ncells, di, dj);
        int i = ci + di, jj = cj + dj;
        if (i >= 0 && i < a.nx && jj >= 0 && jj < a.ny)
        {
          c = (uint64_t)jj * a.nx + i;
          cb = a.col[2 * c];
          ok = boxMeets(h, cb, a.col[2 * c + 1].x);
        }
      }
      unsigned mask = __ballot_sync(0xffffffffu, ok);
      while (mask && !surrounded)
      {
        int src = __ffs(mask) - 1;
        mask &= mask - 1;
        const uint64_t cc = __shfl_sync(0xffffffffu, c, src);
        if (arcWants(cb, src) && column(cc))
          decide();
      }
    }
  }
#ifdef WB_CLASSIFY_STATS
  const long long tNear = clock64();
  stat[8] += tNear - tStart;
#endif
  // Far field: rings of super-cells (WB_SUPER x WB_SUPER columns) pruned as a
  // block; columns already visited in the near field are skipped.
  const int S = WB_SUPER;
  int si = ci >= 0 ? ci / S : -((-ci + S - 1) / S), sj = cj >= 0 ? cj / S : -((-cj + S - 1) / S);
  const int smax = ps.smax;
  for (int sr = 0; sr <= smax && !surrounded && kmax > kNear; sr++)
  {
    if (si + sr < 0 || si - sr >= a.snx || sj + sr < 0 || sj - sr >= a.sny)
      continue;
    int nsc = sr == 0 ? 1 : 8 * sr;
    WB_STAT(stat[2], nsc);
    for (int m0 = 0; m0 < nsc && !surrounded; m0 += 32)
    {
      int m = m0 + lane;
      int SI = 0, SJ = 0;
      bool ok = false;
      int4 sb = make_int4(0, 0, 0, 0);
      if (m < nsc)
      {
        int di, dj;
        ringCell(sr, m, di, dj);
        SI = si + di;
        SJ = sj + dj;
        if (SI >= 0 && SI < a.snx && SJ >= 0 && SJ < a.sny)
        {
          const uint64_t sc = (uint64_t)SJ * a.snx + SI;
          sb = a.super[2 * sc];
          ok = boxMeets(h, sb, a.super[2 * sc + 1].x);
        }
      }
      unsigned mask = __ballot_sync(0xffffffffu, ok);
      while (mask && !surrounded)
      {
        int src = __ffs(mask) - 1;
        mask &= mask - 1;
        const int SIs = __shfl_sync(0xffffffffu, SI, src), SJs = __shfl_sync(0xffffffffu, SJ, src);
        if (!arcWants(sb, src))
          continue;
        int bi = SIs * S, bj = SJs * S;
        // lanes 0..S*S-1 take the block's columns
        uint64_t c = 0;
        bool cok = false;
        int4 cb = make_int4(0, 0, 0, 0);
        if (lane < S * S)
        {
          int i = bi + lane % S, jj = bj + lane / S;
          int cheb = max(abs(i - ci), abs(jj - cj));
          if (i < a.nx && jj < a.ny && cheb > kNear)
          {
            c = (uint64_t)jj * a.nx + i;
            cb = a.col[2 * c];
            cok = boxMeets(h, cb, a.col[2 * c + 1].x);
          }
        }
        unsigned cm = __ballot_sync(0xffffffffu, cok);
        WB_STAT(stat[3], S * S);
        bool gotAny = false;
        while (cm)
        {
          int cs = __ffs(cm) - 1;
          cm &= cm - 1;
          const uint64_t cc = __shfl_sync(0xffffffffu, c, cs);
          if (arcWants(cb, cs))
            gotAny |= column(cc);
        }
        if (gotAny)
          decide();
      }
    }
  }
#ifdef WB_CLASSIFY_STATS
  const long long tFar = clock64();
  stat[9] += tFar - tNear;
#endif
  if (!surrounded && ((fast && !a.fp32Only) || a.margin))
  {
    int nocc;
    __syncwarp();
    uint32_t gap = largestGap(bminW, bmaxW, lane, nocc);
    ambiguous = fast && !a.fp32Only && nocc >= 2 && gap < (uint32_t)WB_DEG144 + 2 * kMargin;
    gapNow = gap;
    gapValid = nocc >= 2;
    if (nocc == 1)
    {
      // every direction in one bin: the gap is the rest of the circle
      const bool mine0 = bminW[lane] != 0xffffffffu, mine1 = bminW[lane + 32] != 0xffffffffu;
      const unsigned who = __ballot_sync(0xffffffffu, mine0 || mine1);
      const int src = __ffs(who) - 1;
      const int b = __shfl_sync(0xffffffffu, mine0 ? lane : lane + 32, src);
      const uint32_t mn = bminW[b], mx = bmaxW[b];
      gapNow = (mn - mx) & 0x7fffffffu;
      gapValid = mn != mx;
    }
  }
#ifdef WB_CLASSIFY_STATS
  stat[10] += clock64() - tFar;
  stat[11] += clock64() - tStart;
  if (lane == 0 && !EXACT)
  {
    int L = surrounded ? 1 : 2;
    atomicAdd(&gClassifyStats[L][0], 1ull);
    for (int q = 1; q < 16; q++)
      atomicAdd(&gClassifyStats[L][q], stat[q]);
  }
#endif
  if (lane == 0)
  {
    a.label[j] = surrounded ? 1 : 2;
    if (a.margin)
      a.margin[j] = marginDeg(gapNow, gapValid);
    if (ambiguous)
      a.ambList[atomicAdd(a.ambCount, 1u)] = (uint32_t)j;
  }
}


/* ---- Column groups: one warp classifies up to 32 points of one column,
 * one lane per point ----
 *
 * The points of a grid column share their neighbourhood, so the warp walks
 * the columns around the group once: every column and super-cell is tested
 * against the group's envelope (the highest hyperboloid apex of its points,
 * the smallest polar radius, the column's box as the points' position), and
 * every candidate read is tested by all lanes against their own points
 * (candidates are staged in shared memory and broadcast).  Each lane keeps
 * its own direction extremes in 8 bins of 45 degrees: a gap of 144 degrees
 * cannot hide inside a bin, so the largest gap formed from the bins' extremes
 * is the exact largest gap of the lane's directions, up to the FP32 direction
 * error (kMargin), exactly as in the one-point kernel.  A lane stops testing
 * once its point is proven surrounded; the group ends when every lane has or
 * the neighbourhood is exhausted.  Envelope tests and height bounds are
 * conservative, so a lane that ends unsurrounded has seen every point inside
 * its hyperboloid.  Clouds whose record differences do not fit FP32 send
 * every point to the exact pass instead. */
constexpr int kGroupBins = 8;
constexpr int kGroupColumns = 128;   // columns a group reads before it hands its undecided points over

struct GroupSmem
{
  int4 cand[32];
  uint32_t bmin[kGroupBins][32], bmax[kGroupBins][32];
  /* each lane's open arc of directions that can still change its decision:
     rays e0 = (ex0, ey0) and e1 = (ex1, ey1), widened beyond the gap's ends;
     amode 0: every direction counts, 1: the wedge from e0 to e1
     counter-clockwise (narrower than a half turn), 2: everything except the
     wedge from e1 to e0 */
  float ex0[32], ey0[32], ex1[32], ey1[32];
  int amode[32];
  uint32_t gapAt[32];   /* a lane's largest gap when its point was proven surrounded */
  /* per lane: store position, reach in column rings and super-cell rings */
  uint32_t j[32];
  int kmax[32], smax[32];
  /* the warp's envelope and its column's box (the same for every lane) */
  float apex, por2min;
  int kmaxG, smaxG;
  int4 cbox;
  /* the columns / super-cells the lanes hold while the warp walks them, and
     their boxes (read by every lane from shared memory, not kept in registers) */
  int4 nbox[32], sbox[32];
  unsigned long long ncol[32];
  int2 sij[32];
};


/* Can a box {x0 <= x <= x1, y0 <= y <= y1} (metres from the point) hold a
 * direction inside the lane's arc?  The largest (smallest) value of a linear
 * form over a box is the sum of its two per-axis extremes. */
__device__ __forceinline__ bool arcMeetsBox(const GroupSmem &sm, int lane, float x0, float x1, float y0, float y1)
{
  const int m = sm.amode[lane];
  if (m == 0)
    return true;
  const float e0x = sm.ex0[lane], e0y = sm.ey0[lane], e1x = sm.ex1[lane], e1y = sm.ey1[lane];
  if (m == 1)
  {
    const float A = fmaxf(e0x * y0, e0x * y1) + fmaxf(-e0y * x0, -e0y * x1);   // max cross(e0, c)
    const float B = fmaxf(e1y * x0, e1y * x1) + fmaxf(-e1x * y0, -e1x * y1);   // max cross(c, e1)
    const float bx = e0x + e1x, by = e0y + e1y;                                // the wedge's bisector
    const float D = fmaxf(bx * x0, bx * x1) + fmaxf(by * y0, by * y1);
    return A >= 0.f && B >= 0.f && D >= 0.f;
  }
  const float A = fminf(e1x * y0, e1x * y1) + fminf(-e1y * x0, -e1y * x1);     // min cross(e1, c)
  const float B = fminf(e0y * x0, e0y * x1) + fminf(-e0x * y0, -e0x * y1);     // min cross(c, e0)
  return !(A > 0.f && B > 0.f);   // the box lies inside the complement wedge from e1 to e0
}

/* The lane's arc from its largest gap (u0 counter-clockwise over w units). */
__device__ __forceinline__ void setArc(GroupSmem &sm, int lane, uint32_t u0, uint32_t w)
{
  const float a0 = (float)u0 * kUnitRad - kArcPad;
  const float W = (float)w * kUnitRad + 2.f * kArcPad;
  if (!(W < 6.2f))
  {
    sm.amode[lane] = 0;
    return;
  }
  float s0, c0, s1, c1;
  // the fast intrinsics are accurate to 4e-7 on [-pi, pi], far inside kArcPad
  const float a1 = a0 + W;
  __sincosf(a0 > 3.14159265f ? a0 - 6.28318531f : a0, &s0, &c0);
  __sincosf(a1 > 3.14159265f ? (a1 > 9.42477796f ? a1 - 12.56637061f : a1 - 6.28318531f) : a1, &s1, &c1);
  sm.ex0[lane] = c0;
  sm.ey0[lane] = s0;
  sm.ex1[lane] = c1;
  sm.ey1[lane] = s1;
  sm.amode[lane] = W < 3.14159f ? 1 : 2;
}

__device__ __forceinline__ void classifyGroup(const ClsArgs &a, uint2 grp, int lane, GroupSmem &sm)
{
  const uint64_t col = grp.x;
  const int4 cbox = a.col[2 * col], cr1 = a.col[2 * col + 1];
  const uint32_t ce = (uint32_t)cr1.z;
  const int ci0 = (int)(col % (uint64_t)a.nx), cj0 = (int)(col / (uint64_t)a.nx);
  const float sx = a.fsx, sy = a.fsy, sz = a.fsz, s2 = a.fs2;
  const int32_t oz = cr1.x;   // height origin of the envelope: the column's lowest point
  {
    const uint32_t g = grp.y;
    const uint32_t t = g + lane;
    bool act = false;
    int4 me = make_int4(0, 0, 0, 0);
    PtSetup ps{};
    uint32_t j = 0;
    if (t < ce)
    {
      me = a.gpt[t];
      j = (uint32_t)me.w & 0x7fffffffu;
      if (a.owner[j] >= 0)
      {
        act = true;
        ps = a.setup[j];
      }
      else
      {
        a.label[j] = 0;
        if (a.margin)
          a.margin[j] = __int_as_float(0x7fc00000);
      }
    }
    if (!__any_sync(0xffffffffu, act))
      return;
#ifdef WB_CLASSIFY_STATS
    const long long tG = clock64();
    unsigned long long gst[16] = {0};
#endif
    if (!a.exactInts)
    {
      // FP32 differences are not exact for this cloud: the exact pass decides
      if (act)
      {
        a.label[j] = 2;
        a.ambList[atomicAdd(a.ambCount, 1u)] = j;
      }
      return;
    }
    for (int b = 0; b < kGroupBins; b++)
    {
      sm.bmin[b][lane] = 0xffffffffu;
      sm.bmax[b][lane] = 0;
    }
    sm.amode[lane] = 0;
    unsigned occ = 0;
    bool done = !act;
    // The envelope of the lanes still undecided: highest apex above oz,
    // smallest polar radius, reach in rings.  It is formed again after every
    // column read, so it shrinks as lanes are decided (a tall point proven
    // surrounded no longer widens the search of the low ones).
    {
      const int offG = max(abs(ps.ci - ci0), abs(ps.cj - cj0));
      sm.kmax[lane] = ps.kmax + offG;
      sm.smax[lane] = ps.smax + (offG + WB_SUPER - 1) / WB_SUPER + 1;
      sm.j[lane] = j;
      if (lane == 0)
        sm.cbox = cbox;
    }
    const float czp = ps.czp, por2 = ps.por2f;
    // the envelope's values live in shared memory (one copy per warp)
    auto envelope = [&]() {
      float ap = !done ? (float)(me.z - oz) * sz + czp : -INFINITY;
      float pm = !done ? por2 : INFINITY;
      int km = !done ? sm.kmax[lane] : 0;
      int sg = !done ? sm.smax[lane] : 0;
      for (int o = 16; o; o >>= 1)
      {
        ap = fmaxf(ap, __shfl_xor_sync(0xffffffffu, ap, o));
        pm = fminf(pm, __shfl_xor_sync(0xffffffffu, pm, o));
        km = max(km, __shfl_xor_sync(0xffffffffu, km, o));
        sg = max(sg, __shfl_xor_sync(0xffffffffu, sg, o));
      }
      __syncwarp();
      if (lane == 0)
      {
        sm.apex = ap;
        sm.por2min = pm;
        sm.kmaxG = km;
        sm.smaxG = sg;
      }
      __syncwarp();
    };
    envelope();
    bool deferred = false;
    int columnsRead = 0;
#ifdef WB_CLASSIFY_STATS
    bool farField = false;   // lane tests beyond the near field (instrumented builds)
#endif
    // envelope test of a box {x0, y0, x1, y1} with lowest point zmin
    auto envMeets = [&](const int4 &b, int32_t zmin) -> bool {
      if (b.x == INT32_MAX)
        return false;
      const int4 cb0 = sm.cbox;
      const float apex = sm.apex, por2min = sm.por2min;
      float dx = (float)max(0, max(b.x - cb0.z, cb0.x - b.z)) * sx;
      float dy = (float)max(0, max(b.y - cb0.w, cb0.y - b.w)) * sy;
      float zd = apex - (float)(zmin - oz) * sz;
      float r2 = s2 * (dx * dx + dy * dy);
      float mag = zd * zd + r2 + por2min;
      if (zd < -1e-4f * (fabsf(zd) + 1e-3f))
        return false;
      return zd * zd - r2 - por2min >= -(1e-4f * mag + 1e-9f);
    };
    // height (record units above oz) above which no point of a column can be
    // inside any lane's hyperboloid; columns holding points outside the root
    // cube in x or y get no bound
    auto envZlim = [&](const int4 &b, const int4 &r1) -> int32_t {
      if (r1.w || !(sz > 0))
        return INT32_MAX;
      const int4 cb0 = sm.cbox;
      const float apex = sm.apex, por2min = sm.por2min;
      float dx = (float)max(0, max(b.x - cb0.z, cb0.x - b.z)) * sx;
      float dy = (float)max(0, max(b.y - cb0.w, cb0.y - b.w)) * sy;
      float need = sqrtf(por2min + s2 * (dx * dx + dy * dy));
      float dz = (apex - need + 1e-4f * (fabsf(apex) + need) + 1e-6f) / sz + 2.f;
      return dz > 2.1e9f ? INT32_MAX : (dz < -2.1e9f ? INT32_MIN : (int32_t)floorf(dz));
    };
    // the lane's surround test from its bins.  A gap below the decision
    // threshold can never decide the lane, so directions that can only fall
    // into such gaps change nothing: when one gap alone is wide enough to
    // matter, the lane's arc is that gap, and boxes outside it are skipped.
    auto decideLane = [&](uint32_t &worst) -> bool {
      worst = 0;
      if (__popc(occ) < 2)
        return false;
      const uint32_t thr = a.fp32Only ? (uint32_t)WB_DEG144 : (uint32_t)WB_DEG144 - 2 * kMargin;
      uint32_t g0 = 0, gw = 0;
      int nbig = 0;
      for (int b = 0; b < kGroupBins; b++)
        if ((occ >> b) & 1)
        {
          unsigned rest = occ >> (b + 1);
          int nb = rest ? b + __ffs(rest) : __ffs(occ) - 1;
          const uint32_t u0 = sm.bmax[b][lane];
          const uint32_t gap = (sm.bmin[nb][lane] - u0) & 0x7fffffffu;
          worst = max(worst, gap);
          if (gap >= thr)
          {
            nbig++;
            g0 = u0;
            gw = gap;
          }
        }
      const bool dec = a.fp32Only ? worst < (uint32_t)WB_DEG144 : worst + 2 * kMargin < (uint32_t)WB_DEG144;
      if (dec)
        sm.gapAt[lane] = worst;
      if (!dec && nbig == 1)
        setArc(sm, lane, g0, gw);
      else
        sm.amode[lane] = 0;
      return dec;
    };
    // whether any undecided lane's arc meets box src of boxes (shared memory)
    // (record integers); true at once while no undecided lane has an arc
    auto boxWanted = [&](const int4 *boxes, int src) -> bool {
      if (!__any_sync(0xffffffffu, !done && sm.amode[lane] != 0))
        return true;
      const int4 b = boxes[src];
      bool want = false;
      if (!done)
        want = arcMeetsBox(sm, lane, (float)(b.x - me.x) * sx, (float)(b.z - me.x) * sx, (float)(b.y - me.y) * sy,
                           (float)(b.w - me.y) * sy);
      return __any_sync(0xffffffffu, want);
    };
    // reads column cc's candidates below the envelope's height bound, each
    // tested by every lane still undecided
    auto scanColumn = [&](uint64_t cc) {
      WB_STAT(gst[1], 1);
#ifdef WB_CLASSIFY_STATS
      const long long tCol = clock64();
#endif
      columnsRead++;
      const int4 box = a.col[2 * cc], r1 = a.col[2 * cc + 1];
      const uint32_t e = (uint32_t)r1.z;
      const int32_t zl = envZlim(box, r1);
      bool got = false;
      // whether candidate c is inside the lane's hyperboloid, in FP32: 1
      // inside, 0 outside (or no direction), 2 when the exact test decides
      // (points outside the root cube, and the band where FP32 cannot tell);
      // dx, dy its offset for the direction.  Fused multiply-adds only
      // make the FP32 values closer to the exact ones, well inside the 1e-5
      // relative tolerances.
      auto memberFast = [&](const int4 &c, float &dx, float &dy) -> int {
        const int32_t dxi = c.x - me.x, dyi = c.y - me.y;
        dx = (float)dxi * sx;
        dy = (float)dyi * sy;
        const uint32_t gp = (uint32_t)c.w;
        const float dzm = (float)(me.z - c.z) * sz;
        const float zd = dzm + czp;
        const float r2 = s2 * __fmaf_rn(dx, dx, dy * dy);
        const float f = __fmaf_rn(zd, zd, -r2) - por2;
        const float tol = __fmaf_rn(1e-5f, __fmaf_rn(zd, zd, r2) + por2, 1e-12f);
        const float ztol = __fmaf_rn(1e-5f, fabsf(dzm) + fabsf(czp), 1e-12f);
        const bool sureIn = zd > ztol && f > tol, sureOut = zd < -ztol || f < -tol;
        int m = sureIn ? 1 : 0;
        if ((gp & kStray) || (!sureIn && !sureOut))
          m = (!(gp & kStray) && a.fp32Only) ? (zd > 0 && f > 0 ? 1 : 0) : 2;
        // dist(p,q) == 0 gives no direction (classify.cpp:142,153)
        return (dxi != 0 || dyi != 0) ? m : 0;
      };
      auto addDir = [&](uint32_t u) {
        const int bin = (int)(u >> 28);
        sm.bmin[bin][lane] = min(sm.bmin[bin][lane], u);
        sm.bmax[bin][lane] = max(sm.bmax[bin][lane], u);
        occ |= 1u << bin;
        got = true;
      };
      for (uint32_t t0 = (uint32_t)r1.y; t0 < e; t0 += 32)
      {
        int4 q = make_int4(0, 0, 0, 0);
        bool low = false, keep = false;
        if (t0 + lane < e)
        {
          q = a.gpt[t0 + lane];
          low = zl == INT32_MAX || q.z - oz <= zl;
          // can q be inside the hyperboloid of any undecided lane?  (its own
          // distance to the group's column; points outside the root cube are
          // left to the exact test)
          keep = low;
          if (low && !((uint32_t)q.w & kStray))
          {
            const int4 cb0 = sm.cbox;
            const float apex = sm.apex, por2min = sm.por2min;
            float ex = (float)max(0, max(q.x - cb0.z, cb0.x - q.x)) * sx;
            float ey = (float)max(0, max(q.y - cb0.w, cb0.y - q.y)) * sy;
            float zd = apex - (float)(q.z - oz) * sz;
            float r2 = s2 * (ex * ex + ey * ey);
            float mag = zd * zd + r2 + por2min;
            keep = zd >= -1e-4f * (fabsf(zd) + 1e-3f) && zd * zd - r2 - por2min >= -(1e-4f * mag + 1e-9f);
          }
        }
        if (!__any_sync(0xffffffffu, low))
          break;
        unsigned lm = __ballot_sync(0xffffffffu, keep);
        WB_STAT(gst[2], __popc(lm));
        WB_STAT(gst[11], farField ? __popc(lm) * __popc(__ballot_sync(0xffffffffu, !done)) : 0);
        WB_STAT(gst[3], __popc(lm) * __popc(__ballot_sync(0xffffffffu, !done)));
        sm.cand[lane] = q;
        __syncwarp();
#ifdef WB_CLASSIFY_STATS
        const long long tCand = clock64();
#endif
        // Every lane runs the tests (a decided lane's results are dropped), so
        // the warp does not diverge on them; the directions are formed only
        // when some lane has a candidate inside.  Two candidates a step: their
        // FP32 tests and directions are independent, so their latencies
        // overlap (31% faster than one a step; the bins are minima and maxima,
        // so the order of the two updates does not matter).  Four a step
        // measured 35% slower than two (register spills), and testing a whole
        // chunk first and forming the directions afterwards 40% slower than one.
        unsigned pend = 0;   // this lane's candidates of the chunk that need the exact test
        while (lm)
        {
          const int k1 = __ffs(lm) - 1;
          lm &= lm - 1;
          const bool two = lm != 0;
          const int k2 = two ? __ffs(lm) - 1 : k1;
          lm &= lm - 1;
          const int4 c1 = sm.cand[k1], c2 = sm.cand[k2];
          float dx1, dy1, dx2, dy2;
          int m1 = memberFast(c1, dx1, dy1), m2 = memberFast(c2, dx2, dy2);
          // the exact tests wait until the chunk's end (bin updates commute),
          // which keeps the call out of this loop: fewer registers live
          // across it and fewer spills (11% faster)
          if (m1 == 2)
          {
            pend |= 1u << k1;
            m1 = 0;
          }
          if (two && m2 == 2)
          {
            pend |= 1u << k2;
            m2 = 0;
          }
          const bool in1 = m1 != 0 && !done, in2 = two && m2 != 0 && !done;
          const bool a1 = __any_sync(0xffffffffu, in1), a2 = __any_sync(0xffffffffu, in2);
          WB_STAT(gst[9], 1);
          WB_STAT(gst[10], (a1 ? 1 : 0) + (a2 ? 1 : 0));
          WB_STAT(gst[7], __popc(__ballot_sync(0xffffffffu, in1)) + __popc(__ballot_sync(0xffffffffu, in2)));
          if (a1 && a2)
          {
            const float f1 = wb_dir_units_f32(dy1, dx1), f2 = wb_dir_units_f32(dy2, dx2);
            if (in1)
              addDir((uint32_t)__float2int_rn(f1) & 0x7fffffffu);
            if (in2)
              addDir((uint32_t)__float2int_rn(f2) & 0x7fffffffu);
          }
          else if (a1 || a2)
          {
            const float f = a1 ? wb_dir_units_f32(dy1, dx1) : wb_dir_units_f32(dy2, dx2);
            if (in1 || in2)
              addDir((uint32_t)__float2int_rn(f) & 0x7fffffffu);
          }
        }
        while (__any_sync(0xffffffffu, pend != 0))
        {
          bool inE = false;
          float dxE = 0.f, dyE = 0.f;
          if (pend)
          {
            const int kE = __ffs(pend) - 1;
            pend &= pend - 1;
            const int4 cE = sm.cand[kE];
            dxE = (float)(cE.x - me.x) * sx;
            dyE = (float)(cE.y - me.y) * sy;
            inE = !done && memberExact(a, exactHyp(a, sm.j[lane]), (uint32_t)cE.w, cE.x, cE.y, cE.z);
          }
          if (__any_sync(0xffffffffu, inE))
          {
            const float f = wb_dir_units_f32(dyE, dxE);
            if (inE)
              addDir((uint32_t)__float2int_rn(f) & 0x7fffffffu);
          }
        }
        __syncwarp();
#ifdef WB_CLASSIFY_STATS
        gst[14] += clock64() - tCand;
#endif
      }
#ifdef WB_CLASSIFY_STATS
      const long long tDec = clock64();
#endif
      uint32_t worst;
      if (got && !done)
        done = decideLane(worst);
#ifdef WB_CLASSIFY_STATS
      gst[15] += clock64() - tDec;
#endif
#ifdef WB_CLASSIFY_STATS
      const long long tEnv = clock64();
      gst[12] += tEnv - tCol;
#endif
      if (__any_sync(0xffffffffu, got))
        envelope();
#ifdef WB_CLASSIFY_STATS
      gst[13] += clock64() - tEnv;
#endif
    };
    // A group whose neighbourhood is very large would hold one warp while the
    // rest of the GPU idles: after kGroupColumns columns its undecided points
    // go to the one-point kernel.  (Handing over a group with few lanes left
    // as well measured 11% slower with these limits: 6 lanes, 256 columns.)
    auto allDone = [&]() {
      if (__all_sync(0xffffffffu, done))
        return true;
      if (columnsRead <= kGroupColumns)
        return false;
      if (!done)
      {
        deferred = true;
        done = true;
        a.deferList[atomicAdd(a.deferCount, 1u)] = sm.j[lane];
      }
      return true;
    };
    // near field: the group's column and the ring around it
    const int kNearG = 1;   // one ring of single columns (none: 5% slower, two: 1% slower)
    for (int ring = 0; ring <= kNearG && ring <= sm.kmaxG && !allDone(); ring++)
    {
      const int ncells = ring == 0 ? 1 : 8 * ring;
      const int stride = ring == 0 ? 1 : 4 * ring - 1;
      uint64_t c = 0;
      bool ok = false;
      int4 cb = make_int4(0, 0, 0, 0);
      if (lane < ncells)
      {
        int di, dj;
        ringCell(ring, (lane * stride) % ncells, di, dj);
        int i = ci0 + di, jj = cj0 + dj;
        if (i >= 0 && i < a.nx && jj >= 0 && jj < a.ny)
        {
          c = (uint64_t)jj * a.nx + i;
          cb = a.col[2 * c];
          ok = envMeets(cb, a.col[2 * c + 1].x);
        }
      }
      unsigned mask = __ballot_sync(0xffffffffu, ok);
      __syncwarp();
      sm.nbox[lane] = cb;
      sm.ncol[lane] = c;
      __syncwarp();
      while (mask && !allDone())
      {
        const int src = __ffs(mask) - 1;
        mask &= mask - 1;
        const uint64_t cc = sm.ncol[src];
        if (boxWanted(sm.nbox, src))
          scanColumn(cc);
      }
    }
    // far field: rings of super-cells, then their columns outside the near field
#ifdef WB_CLASSIFY_STATS
    farField = true;
#endif
    const int S = WB_SUPER;
    const int si = ci0 / S, sj = cj0 / S;
    for (int sr = 0; sr <= sm.smaxG && sm.kmaxG > kNearG && !allDone(); sr++)
    {
      if (si + sr < 0 || si - sr >= a.snx || sj + sr < 0 || sj - sr >= a.sny)
        continue;
      const int nsc = sr == 0 ? 1 : 8 * sr;
      for (int m0 = 0; m0 < nsc && !allDone(); m0 += 32)
      {
        const int m = m0 + lane;
        int SI = 0, SJ = 0;
        bool ok = false;
        int4 sb = make_int4(0, 0, 0, 0);
        if (m < nsc)
        {
          int di, dj;
          ringCell(sr, m, di, dj);
          SI = si + di;
          SJ = sj + dj;
          if (SI >= 0 && SI < a.snx && SJ >= 0 && SJ < a.sny)
          {
            const uint64_t sc = (uint64_t)SJ * a.snx + SI;
            sb = a.super[2 * sc];
            ok = envMeets(sb, a.super[2 * sc + 1].x);
          }
        }
        unsigned mask = __ballot_sync(0xffffffffu, ok);
        __syncwarp();
        sm.sbox[lane] = sb;
        sm.sij[lane] = make_int2(SI, SJ);
        __syncwarp();
        while (mask && !allDone())
        {
          const int src = __ffs(mask) - 1;
          mask &= mask - 1;
          const int SIs = sm.sij[src].x, SJs = sm.sij[src].y;
          if (!boxWanted(sm.sbox, src))
            continue;
          const int bi = SIs * S, bj = SJs * S;
          uint64_t c = 0;
          bool cok = false;
          int4 cb = make_int4(0, 0, 0, 0);
          if (lane < S * S)
          {
            const int i = bi + lane % S, jj = bj + lane / S;
            if (i < a.nx && jj < a.ny && max(abs(i - ci0), abs(jj - cj0)) > kNearG)
            {
              c = (uint64_t)jj * a.nx + i;
              cb = a.col[2 * c];
              cok = envMeets(cb, a.col[2 * c + 1].x);
            }
          }
          unsigned cm = __ballot_sync(0xffffffffu, cok);
          __syncwarp();
          sm.nbox[lane] = cb;
          sm.ncol[lane] = c;
          __syncwarp();
          while (cm && !allDone())
          {
            const int cs = __ffs(cm) - 1;
            cm &= cm - 1;
            const uint64_t cc = sm.ncol[cs];
            if (boxWanted(sm.nbox, cs))
              scanColumn(cc);
          }
        }
      }
    }
#ifdef WB_CLASSIFY_STATS
    const unsigned bAct = __ballot_sync(0xffffffffu, act), bDef = __ballot_sync(0xffffffffu, deferred);
    const unsigned bGnd = __ballot_sync(0xffffffffu, act && !deferred && !done);
    if (lane == 0)
    {
      gst[0] = 1;
      gst[4] = __popc(bAct);
      gst[5] = __popc(bDef);
      gst[6] = clock64() - tG;
      gst[8] = __popc(bGnd);

      for (int q = 0; q < 16; q++)
        atomicAdd(&gClassifyStats[0][q], gst[q]);
    }
#endif
    if (act && !deferred)
    {
      const uint32_t j = sm.j[lane];
      uint32_t worst = 0;
      bool amb = false;
      if (!done)
      {
        decideLane(worst);
        amb = !a.fp32Only && __popc(occ) >= 2 && worst < (uint32_t)WB_DEG144 + 2 * kMargin;
      }
      a.label[j] = done ? 1 : 2;
      if (a.margin)
      {
        if (done)
          a.margin[j] = marginDeg(sm.gapAt[lane], true);
        else if (__popc(occ) == 1)
        {
          // every direction in one bin: the gap is the rest of the circle
          const int b = __ffs(occ) - 1;
          const uint32_t mn = sm.bmin[b][lane], mx = sm.bmax[b][lane];
          a.margin[j] = marginDeg((mn - mx) & 0x7fffffffu, mn != mx);
        }
        else
          a.margin[j] = marginDeg(worst, __popc(occ) >= 2);
      }
      if (amb)
        a.ambList[atomicAdd(a.ambCount, 1u)] = j;
    }
  }
}
}  // namespace

/* Decoding is strictly increasing in every record integer when the step
 * scale*unit is at least four ulps of every coordinate the root cube spans;
 * then equal decoded doubles mean equal integers, and FP32 differences of
 * integers stand for differences of the doubles. */
static bool decodeIsExact(const WbGeom &g, const double mn[3], const double mx[3])
{
  // the decode must increase with the record integer (the FP32 paths take a
  // box's low record integers as its low coordinates and a column's height
  // order from its record order), in steps FP64 resolves
  for (int a = 0; a < 3; a++)
  {
    double step = g.scale[a] * g.unit;
    double mag = fmax(fabs(mn[a]), fabs(mx[a])) + fabs(g.off[a] * g.unit) + step;
    if (!(step > 0) || step < 4 * ldexp(mag, -52))
      return false;
  }
  return true;
}

/* Checks the state, sizes the buffers, uploads the angle tables and the
 * incoming class bytes, and forms the kernel arguments (on c's stream). */
static int classifyPrepare(wb_ctx *c, const wb_params *p, uint8_t *cls, int onDevice, ClsArgs &a)
{
  if (c->stage < 2)
    return wb_fail(c, WB_ESTATE, "wb_classify: scan the tiles first");
  if (!cls && c->n)
    return wb_fail(c, WB_EINVAL, "wb_classify: cls must not be NULL");
  if (!(p->max_slope > 0))
    return wb_fail(c, WB_EINVAL, "wb_classify: max_slope must be > 0");
  if (onDevice && c->n && !wb_device_accessible(cls))
    return wb_fail(c, WB_EINVAL, "wb_classify: device class bytes must be device memory");
  int rc;
  uint64_t nd = c->nd, n = c->n;
  if ((rc = wb_ensure(c, c->label, nd + 64)) || (rc = wb_ensure(c, c->angleT, (511 + 512 + 512) * 8)) ||
      (rc = wb_ensure(c, c->ambiguous, nd * 4 + 64)) || (rc = wb_ensure(c, c->ptSetup, nd * sizeof(PtSetup) + 64)) ||
      (rc = wb_ensure(c, c->deferred, nd * 4 + 64)))
    return rc;
  if (!onDevice && (rc = wb_ensure(c, c->clsDev, n + 64)))
    return rc;
  double *tab = (double *)c->angleT.p;
  WB_CUDA(c, cudaMemcpyAsync(tab, kWbTan, 511 * 8, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaMemcpyAsync(tab + 511, kWbSin, 512 * 8, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaMemcpyAsync(tab + 1023, kWbCos, 512 * 8, cudaMemcpyDefault, c->stream));
  uint8_t *clsDev = onDevice ? cls : (uint8_t *)c->clsDev.p;
  if (!onDevice && n && (rc = wb_copy_in(c, clsDev, cls, n)))
    return rc;
  wb_mark(c, "cls_upload");
  a.nd = nd;
  const WbGeom &g = c->g;
  double mn[3], mx[3];
  for (int k = 0; k < 3; k++)
  {
    a.off[k] = g.off[k];
    a.scale[k] = g.scale[k];
    a.rootLo[k] = g.root_lo[k];
    mn[k] = g.root_lo[k];
    mx[k] = g.root_lo[k] + g.root_side;
  }
  a.unit = g.unit;
  a.slope = p->max_slope;
  a.thickness = p->thickness;
  a.leafKey = (const uint64_t *)c->leafKey.p;
  a.leafLev = (const uint8_t *)c->leafLevel.p;
  a.leafId = (const uint32_t *)c->leafId.p;
  a.rootSide = g.root_side;
  a.sx = (const int32_t *)c->sx.p;
  a.sy = (const int32_t *)c->sy.p;
  a.sz = (const int32_t *)c->sz.p;
  a.xyzd = (const double *)c->xyzd.p;
  a.owner = (const int32_t *)c->owner.p;
  a.tiles = (const TileRes *)c->tileRes.p;
  a.tanT = tab;
  a.sinT = tab + 511;
  a.cosT = tab + 1023;
  a.label = (uint8_t *)c->label.p;
  a.gx0 = c->grid.x0;
  a.gy0 = c->grid.y0;
  a.cell = c->grid.cell;
  a.invSlope2 = 1.0 / (p->max_slope * p->max_slope);
  a.invCellF = (float)(1.0 / c->grid.cell);
  a.invSuperF = (float)(1.0 / (WB_SUPER * c->grid.cell));
  a.colOf = (const int2 *)c->colOf.p;
  a.nx = c->grid.nx;
  a.ny = c->grid.ny;
  a.ncell = c->grid.ncell;
  a.col = (const int4 *)c->cellRec.p;
  a.gpt = (const int4 *)c->gpt.p;
  a.groups = (const uint2 *)c->groups.p;
  a.snx = c->grid.snx;
  a.sny = c->grid.sny;
  a.super = (const int4 *)c->superRec.p;
  a.zmin = (g.off[2] + g.scale[2] * (double)c->grid.zminInt) * g.unit;
  bool fits32 = true;
  for (int k = 0; k < 3; k++)
    fits32 = fits32 && (int64_t)c->grid.imax[k] - (int64_t)c->grid.imin[k] < ((int64_t)1 << 30);
  a.exactInts = (decodeIsExact(g, mn, mx) && fits32) ? 1 : 0;
  a.fp32Only = (c->precision == WB_PRECISION_FP32 && a.exactInts) ? 1 : 0;
  a.fsx = (float)(g.scale[0] * g.unit);
  a.fsy = (float)(g.scale[1] * g.unit);
  a.fsz = (float)(g.scale[2] * g.unit);
  a.fs2 = (float)(p->max_slope * p->max_slope);
  a.setup = (PtSetup *)c->ptSetup.p;
  a.ambList = (uint32_t *)c->ambiguous.p;
  a.ambCount = (uint32_t *)((char *)c->small.p + 448);
  a.deferList = (uint32_t *)c->deferred.p;
  a.deferCount = (uint32_t *)((char *)c->small.p + 452);
  a.work = nullptr;
  a.nwork = 0;
  a.n = n;
  a.nTiles = c->n_tiles;
  a.storeOf = (const uint32_t *)c->storeOf.p;
  a.cls = clsDev;
  a.margin = a.marginOut = nullptr;
  if (c->marginDst)
  {
    if ((rc = wb_ensure(c, c->marginBuf, nd * 4 + 64)))
      return rc;
    a.margin = (float *)c->marginBuf.p;
    if (onDevice)
      a.marginOut = c->marginDst;
    else
    {
      if ((rc = wb_ensure(c, c->marginRec, n * 4 + 64)))
        return rc;
      a.marginOut = (float *)c->marginRec.p;
    }
  }
  WB_CUDA(c, cudaMemsetAsync(a.ambCount, 0, 8, c->stream));   // ambiguous and deferred counts
  return 0;
}

/* ---- Fused classify of many jobs: one persistent launch over all their points ----
 *
 * Each job is a context that has been built and scanned; wb_classify_stage
 * formed its kernel arguments.  The job table (arguments and prefix sums of
 * the jobs' point, record and tile counts) is uploaded from a pinned mirror
 * by the first node of a captured CUDA graph, so one graph serves every
 * batch: the kernels read the job count and offsets from device memory.
 * Warps of the persistent ring kernel take chunks of consecutive points from
 * a global counter and copy the owning job's arguments to shared memory when
 * the job changes. */
namespace
{
struct BatchHdr
{
  int k, chunk;
  unsigned long long next[3];   /* work counters: fast pass, deferred points, exact pass */
  uint64_t startNd[WB_BATCH_MAX + 1], startN[WB_BATCH_MAX + 1], startT[WB_BATCH_MAX + 1];
  uint64_t startGrp[WB_BATCH_MAX + 1];   /* column groups (the column-group fast pass) */
  ClsArgs jobs[WB_BATCH_MAX];
};
struct BatchOut
{
  uint64_t startAmb[WB_BATCH_MAX + 1];   /* prefix of the jobs' ambiguous counts */
  uint64_t startDef[WB_BATCH_MAX + 1];   /* prefix of the jobs' deferred counts */
  unsigned long long ground[WB_BATCH_MAX];
};

/* The job q with start[q] <= g < start[q+1] (start non-decreasing, g < start[k]). */
__device__ __forceinline__ int batchJob(const uint64_t *start, int k, uint64_t g)
{
  int lo = 0, hi = k;
  while (hi - lo > 1)
  {
    int mid = (lo + hi) >> 1;
    if (start[mid] <= g)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

__global__ void batchSetup(const BatchHdr *__restrict__ h)
{
  const int k = h->k;
  const uint64_t total = h->startNd[k];
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (uint64_t)gridDim.x * blockDim.x)
  {
    int q = batchJob(h->startNd, k, g);
    setupPoint(h->jobs[q], g - h->startNd[q]);
  }
}

/* MODE 0: every point of every job; 1: the points column groups deferred;
 * 2: the ambiguous points (exact pass). */
template <int MODE, int W, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) batchRings(BatchHdr *h, const BatchOut *o)
{
  constexpr bool EXACT = MODE == 2;
  __shared__ uint32_t bmin[W][kBins], bmax[W][kBins];
  __shared__ ClsArgs sa[W];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int k = h->k;
  const uint64_t *start = MODE == 2 ? o->startAmb : (MODE == 1 ? o->startDef : h->startNd);
  const uint64_t total = start[k];
  const unsigned chunk = MODE == 0 ? (unsigned)h->chunk : 1u;
  uint64_t lo = 1, hi = 0;
  for (;;)
  {
    unsigned long long base = 0;
    if (lane == 0)
      base = atomicAdd(&h->next[MODE], (unsigned long long)chunk);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total)
      break;
    uint64_t end = base + chunk < total ? base + chunk : total;
    for (uint64_t g = base; g < end; g++)
    {
      if (g < lo || g >= hi)
      {
        int q = batchJob(start, k, g);
        lo = start[q];
        hi = start[q + 1];
        __syncwarp();
        const uint32_t *src = (const uint32_t *)&h->jobs[q];
        uint32_t *dst = (uint32_t *)&sa[w];
        for (int i = lane; i < (int)(sizeof(ClsArgs) / 4); i += 32)
          dst[i] = src[i];
        __syncwarp();
      }
      const ClsArgs &a = sa[w];
      uint64_t item = g - lo;
      classifyPoint<EXACT>(a, MODE == 2 ? a.ambList[item] : (MODE == 1 ? a.deferList[item] : item), lane, bmin[w],
                           bmax[w]);
    }
  }
}

/* The fast pass by column groups: warps take chunks of groups (of all jobs)
 * from a global counter. */
template <int W, int MINB>
__global__ void __launch_bounds__(32 * W, MINB) batchGroups(BatchHdr *h, const BatchOut *o)
{
  __shared__ GroupSmem gsm[W];
  __shared__ ClsArgs sa[W];
  (void)o;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int k = h->k;
  const uint64_t *start = h->startGrp;
  const uint64_t total = start[k];
  const unsigned chunk = (unsigned)h->chunk;
  uint64_t lo = 1, hi = 0;
  for (;;)
  {
    unsigned long long base = 0;
    if (lane == 0)
      base = atomicAdd(&h->next[0], (unsigned long long)chunk);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total)
      break;
    uint64_t end = base + chunk < total ? base + chunk : total;
    for (uint64_t g = base; g < end; g++)
    {
      if (g < lo || g >= hi)
      {
        int q = batchJob(start, k, g);
        lo = start[q];
        hi = start[q + 1];
        __syncwarp();
        const uint32_t *src = (const uint32_t *)&h->jobs[q];
        uint32_t *dst = (uint32_t *)&sa[w];
        for (int i = lane; i < (int)(sizeof(ClsArgs) / 4); i += 32)
          dst[i] = src[i];
        __syncwarp();
      }
      classifyGroup(sa[w], sa[w].groups[g - lo], lane, gsm[w]);
    }
  }
}

/* Prefix of the jobs' deferred (which = 0) or ambiguous (which = 1) counts. */
__global__ void batchPrefix(const BatchHdr *__restrict__ h, BatchOut *__restrict__ o, int which)
{
  if (threadIdx.x || blockIdx.x)
    return;
  uint64_t *out = which ? o->startAmb : o->startDef;
  uint64_t s = 0;
  for (int q = 0; q < h->k; q++)
  {
    out[q] = s;
    s += which ? *h->jobs[q].ambCount : *h->jobs[q].deferCount;
  }
  out[h->k] = s;
}

__global__ void batchZeroGround(const BatchHdr *__restrict__ h, BatchOut *__restrict__ o)
{
  const int k = h->k;
  const uint64_t total = h->startT[k];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < k; q += gridDim.x * blockDim.x)
    o->ground[q] = 0;
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (uint64_t)gridDim.x * blockDim.x)
  {
    int q = batchJob(h->startT, k, g);
    ((TileRes *)h->jobs[q].tiles)[g - h->startT[q]].nGround = 0;
  }
}

__global__ void batchGroundCount(const BatchHdr *__restrict__ h, BatchOut *__restrict__ o)
{
  const int k = h->k;
  const uint64_t total = h->startNd[k];
  const int lane = threadIdx.x & 31;
  // whole warps step together, so the ground points of a warp are counted
  // with one atomic per tile and one per job
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w0 = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); w0 < total; w0 += stride)
  {
    const uint64_t g = w0 + lane;
    bool gnd = false;
    int q = 0;
    int32_t t = -1;
    if (g < total)
    {
      q = batchJob(h->startNd, k, g);
      const ClsArgs &a = h->jobs[q];
      const uint64_t j = g - h->startNd[q];
      t = a.owner[j];
      gnd = t >= 0 && a.label[j] == 2;
    }
    const unsigned m = __ballot_sync(0xffffffffu, gnd);
    if (gnd)
    {
      const unsigned sameT = __match_any_sync(m, ((unsigned long long)q << 32) | (uint32_t)t);
      if (lane == __ffs(sameT) - 1)
        atomicAdd(&((TileRes *)h->jobs[q].tiles)[t].nGround, __popc(sameT));
      const unsigned sameQ = __match_any_sync(m, q);
      if (lane == __ffs(sameQ) - 1)
        atomicAdd(&o->ground[q], (unsigned long long)__popc(sameQ));
    }
  }
}

__global__ void batchScatter(const BatchHdr *__restrict__ h)
{
  const int k = h->k;
  const uint64_t total = h->startN[k];
  for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (uint64_t)gridDim.x * blockDim.x)
  {
    int q = batchJob(h->startN, k, g);
    const ClsArgs &a = h->jobs[q];
    uint64_t i = g - h->startN[q];
    uint32_t j = a.storeOf[i];
    if (a.owner[j] >= 0)
      a.cls[i] = a.label[j];
    if (a.marginOut)
      a.marginOut[i] = a.owner[j] >= 0 ? a.margin[j] : __int_as_float(0x7fc00000);
  }
}
}  // namespace

static_assert(sizeof(ClsArgs) <= sizeof(((wb_ctx *)nullptr)->clsArgs), "wb_ctx::clsArgs too small");

struct WbBatch
{
  int device = 0, sm = 0;
  cudaStream_t capture = nullptr;
  BatchHdr *dIn = nullptr, *hIn = nullptr;
  BatchOut *dOut = nullptr, *hOut = nullptr;
  int per[WB_N_SHAPES + 2] = {0};   /* resident blocks per SM of each classify kernel */
  cudaGraphExec_t graphs[WB_N_SHAPES] = {nullptr};
};

const WbShape kWbShapes[WB_N_SHAPES] = {{8, 3}, {4, 5}, {8, 2}, {8, 3}, {4, 6}, {4, 8}, {8, 4}, {2, 12}};

namespace
{
typedef void (*RingsFn)(BatchHdr *, const BatchOut *);

/* Kernels of the fused classify: 0..WB_N_SHAPES-1 the fast pass of each
 * shape (one point per warp, or column groups), kDeferred the one-point pass
 * over the points column groups handed over, kExactPass the exact pass. */
constexpr int kDeferred = WB_N_SHAPES, kExactPass = WB_N_SHAPES + 1;

RingsFn ringsFn(int idx)
{
  // kWbShapes 0-2: column groups (register caps of about 85, 102 and 128 a
  // thread); 3-7: one point per warp (about 85, 85, 64, 64 and 85)
  switch (idx)
  {
  case 1: return batchGroups<4, 5>;
  case 2: return batchGroups<8, 2>;
  case 3: return batchRings<0, 8, 3>;
  case 4: return batchRings<0, 4, 6>;
  case 5: return batchRings<0, 4, 8>;
  case 6: return batchRings<0, 8, 4>;
  case 7: return batchRings<0, 2, 12>;
  case kDeferred: return batchRings<1, 8, 3>;
  case kExactPass: return batchRings<2, 4, 6>;
  default: return batchGroups<8, 3>;
  }
}

int ringsWarps(int idx)
{
  return idx == kExactPass ? 4 : (idx == kDeferred ? 8 : kWbShapes[idx].warps);
}

__global__ void batchAmbReset(const BatchHdr *__restrict__ h)
{
  for (int q = threadIdx.x; q < h->k; q += blockDim.x)
  {
    *h->jobs[q].ambCount = 0;
    *h->jobs[q].deferCount = 0;
  }
}

/* Persistent grid of a ring kernel: every SM filled to its occupancy
 * (queried once; occupancy queries are not stream work, so this also runs
 * before a capture begins). */
cudaError_t ringsGrid(WbBatch *b, int shape, unsigned *grid)
{
  if (!b->per[shape])
  {
    int per = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ringsFn(shape), 32 * ringsWarps(shape), 0);
    if (e != cudaSuccess)
      return e;
    b->per[shape] = per > 0 ? per : 1;
  }
  *grid = (unsigned)(b->sm * b->per[shape]);
  return cudaSuccess;
}

/* The fused classify on stream s: upload of the job table, set-up, the
 * persistent fast pass, the deferred prefix and one-point pass, the ambiguous
 * prefix and exact pass, ground counts (per tile and per job), the
 * class-byte scatter and the read-back of the per-job totals (9 kernels).  With mark, stage events go on mark's stream. */
cudaError_t enqueueBatch(WbBatch *b, cudaStream_t s, int shape, const unsigned grids[3], wb_ctx *mark)
{
  const unsigned grid = (unsigned)b->sm * 8;
  cudaError_t e = cudaMemcpyAsync(b->dIn, b->hIn, sizeof(BatchHdr), cudaMemcpyDefault, s);
  if (e != cudaSuccess)
    return e;
  batchSetup<<<grid, 256, 0, s>>>(b->dIn);
  ringsFn(shape)<<<grids[0], 32 * ringsWarps(shape), 0, s>>>(b->dIn, b->dOut);
  batchPrefix<<<1, 32, 0, s>>>(b->dIn, b->dOut, 0);
  ringsFn(kDeferred)<<<grids[1], 32 * ringsWarps(kDeferred), 0, s>>>(b->dIn, b->dOut);
  if (mark)
    wb_mark(mark, "classify");
  batchPrefix<<<1, 32, 0, s>>>(b->dIn, b->dOut, 1);
  ringsFn(kExactPass)<<<grids[2], 32 * ringsWarps(kExactPass), 0, s>>>(b->dIn, b->dOut);
  if (mark)
    wb_mark(mark, "classify_exact");
  batchZeroGround<<<grid, 256, 0, s>>>(b->dIn, b->dOut);
  batchGroundCount<<<grid, 256, 0, s>>>(b->dIn, b->dOut);
  batchScatter<<<grid, 256, 0, s>>>(b->dIn);
  e = cudaMemcpyAsync(b->hOut, b->dOut, sizeof(BatchOut), cudaMemcpyDefault, s);
  if (e == cudaSuccess)
    e = cudaGetLastError();
  return e;
}

/* The three classify grids of a shape. */
cudaError_t batchGrids(WbBatch *b, int shape, unsigned grids[3])
{
  cudaError_t e = ringsGrid(b, shape, &grids[0]);
  if (e == cudaSuccess)
    e = ringsGrid(b, kDeferred, &grids[1]);
  if (e == cudaSuccess)
    e = ringsGrid(b, kExactPass, &grids[2]);
  return e;
}

cudaError_t captureBatch(WbBatch *b, int shape, cudaGraphExec_t *exec)
{
  unsigned grids[3];
  cudaError_t e = batchGrids(b, shape, grids);
  if (e != cudaSuccess)
    return e;
  cudaGraph_t graph = nullptr;
  e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess)
    return e;
  cudaError_t le = enqueueBatch(b, b->capture, shape, grids, nullptr);
  e = cudaStreamEndCapture(b->capture, &graph);
  if (e == cudaSuccess && le != cudaSuccess)
    e = le;
  if (e == cudaSuccess)
    e = cudaGraphInstantiate(exec, graph, 0);
  if (graph)
    cudaGraphDestroy(graph);
  return e;
}

/* Fills the pinned job table from the staged contexts; with sample > 0 the
 * point ranges are cut after the first `sample` points. */
int fillTable(WbBatch *b, wb_ctx *const *jobs, int k, int chunk, uint64_t sample, std::string &err)
{
  if (k < 1 || k > WB_BATCH_MAX)
  {
    err = "between 1 and " + std::to_string(WB_BATCH_MAX) + " jobs per launch";
    return WB_EINVAL;
  }
  BatchHdr *h = b->hIn;
  h->k = k;
  h->chunk = chunk < 1 ? 1 : chunk;
  h->next[0] = h->next[1] = h->next[2] = 0;
  h->startNd[0] = h->startN[0] = h->startT[0] = h->startGrp[0] = 0;
  for (int q = 0; q < k; q++)
  {
    wb_ctx *c = jobs[q];
    if (!c->clsStaged)
    {
      err = "job " + std::to_string(q) + " was not staged";
      return WB_ESTATE;
    }
    memcpy(&h->jobs[q], c->clsArgs, sizeof(ClsArgs));
    uint64_t nd = c->nd;
    if (sample && h->startNd[q] + nd > sample)
      nd = sample > h->startNd[q] ? sample - h->startNd[q] : 0;
    h->startNd[q + 1] = h->startNd[q] + nd;
    h->startN[q + 1] = h->startN[q] + c->n;
    h->startT[q + 1] = h->startT[q] + c->n_tiles;
    uint64_t ng = c->grid.nGroups;
    if (sample && c->nd)
      ng = (uint64_t)((double)ng * (double)(h->startNd[q + 1] - h->startNd[q]) / (double)c->nd + 0.999);
    h->startGrp[q + 1] = h->startGrp[q] + ng;
  }
  return 0;
}

int clampShape(int shape)
{
  return shape < 0 || shape >= WB_N_SHAPES ? 0 : shape;
}
}  // namespace

int wb_batch_create(int device, WbBatch **out, std::string &err)
{
  *out = nullptr;
  WbBatch *b = new (std::nothrow) WbBatch;
  if (!b)
    return WB_ENOMEM;
  b->device = device;
  WbDeviceGuard deviceGuard(device);
  cudaDeviceGetAttribute(&b->sm, cudaDevAttrMultiProcessorCount, device);
  cudaError_t e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
  if (e == cudaSuccess)
    e = cudaMalloc(&b->dIn, sizeof(BatchHdr));
  if (e == cudaSuccess)
    e = cudaMalloc(&b->dOut, sizeof(BatchOut));
  if (e == cudaSuccess)
    e = cudaMallocHost(&b->hIn, sizeof(BatchHdr));
  if (e == cudaSuccess)
    e = cudaMallocHost(&b->hOut, sizeof(BatchOut));
  if (e != cudaSuccess)
  {
    err = std::string("wb_batch_create: ") + cudaGetErrorString(e);
    cudaGetLastError();
    wb_batch_destroy(b);
    return WB_ENOMEM;
  }
  *out = b;
  return 0;
}

void wb_batch_destroy(WbBatch *b)
{
  if (!b)
    return;
  WbDeviceGuard deviceGuard(b->device);
  for (cudaGraphExec_t g : b->graphs)
    if (g)
      cudaGraphExecDestroy(g);
  if (b->capture)
    cudaStreamDestroy(b->capture);
  cudaFree(b->dIn);
  cudaFree(b->dOut);
  cudaFreeHost(b->hIn);
  cudaFreeHost(b->hOut);
  delete b;
}

int wb_classify_stage(wb_ctx *c, const wb_params *p, uint8_t *cls, int onDevice)
{
  ClsArgs a;
  int rc = classifyPrepare(c, p, cls, onDevice, a);
  if (rc)
    return rc;
  memcpy(c->clsArgs, &a, sizeof a);
  c->clsHost = onDevice ? nullptr : cls;
  c->clsStaged = true;
  return 0;
}

int wb_batch_time(WbBatch *b, wb_ctx *const *jobs, int k, uint64_t sample, int shape, int chunk, cudaStream_t s,
                  float *ms, std::string &err)
{
  shape = clampShape(shape);
  int rc = fillTable(b, jobs, k, chunk, sample, err);
  if (rc)
    return rc;
  WbDeviceGuard deviceGuard(b->device);
  unsigned grids[3];
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = batchGrids(b, shape, grids);
  if (e == cudaSuccess)
    e = cudaEventCreate(&e0);
  if (e == cudaSuccess)
    e = cudaEventCreate(&e1);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->dIn, b->hIn, sizeof(BatchHdr), cudaMemcpyDefault, s);
  if (e == cudaSuccess)
  {
    batchSetup<<<(unsigned)b->sm * 8, 256, 0, s>>>(b->dIn);
    cudaEventRecord(e0, s);
    ringsFn(shape)<<<grids[0], 32 * ringsWarps(shape), 0, s>>>(b->dIn, b->dOut);
    batchPrefix<<<1, 32, 0, s>>>(b->dIn, b->dOut, 0);
    ringsFn(kDeferred)<<<grids[1], 32 * ringsWarps(kDeferred), 0, s>>>(b->dIn, b->dOut);
    cudaEventRecord(e1, s);
    batchAmbReset<<<1, 256, 0, s>>>(b->dIn);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(s);
  if (e == cudaSuccess)
    e = cudaEventElapsedTime(ms, e0, e1);
  if (e0)
    cudaEventDestroy(e0);
  if (e1)
    cudaEventDestroy(e1);
  if (e != cudaSuccess)
  {
    err = std::string("wb_batch_time: ") + cudaGetErrorString(e);
    return WB_ECUDA;
  }
  return 0;
}

int wb_batch_launch(WbBatch *b, wb_ctx *const *jobs, int k, cudaStream_t s, int shape, int chunk,
                    uint64_t *launches, std::string &err)
{
  shape = clampShape(shape);
  int rc = fillTable(b, jobs, k, chunk, 0, err);
  if (rc)
    return rc;
  WbDeviceGuard deviceGuard(b->device);
  if (!b->graphs[shape])
  {
    cudaError_t e = captureBatch(b, shape, &b->graphs[shape]);
    if (e != cudaSuccess)
    {
      cudaGetLastError();
      b->graphs[shape] = nullptr;
      err = std::string("wb_batch_launch: graph capture: ") + cudaGetErrorString(e);
      return WB_ECUDA;
    }
  }
  cudaError_t e = cudaGraphLaunch(b->graphs[shape], s);
  for (int q = 0; q < k && e == cudaSuccess; q++)
  {
    wb_ctx *c = jobs[q];
    ClsArgs *a = (ClsArgs *)c->clsArgs;
    if (c->clsHost && c->n)
      e = cudaMemcpyAsync(c->clsHost, a->cls, c->n, cudaMemcpyDefault, s);
  }
  if (e != cudaSuccess)
  {
    err = std::string("wb_batch_launch: ") + cudaGetErrorString(e);
    return WB_ECUDA;
  }
  if (launches)
    *launches += 9;   /* kernel nodes of the graph */
  return 0;
}

void wb_batch_collect(WbBatch *b, wb_ctx *const *jobs, int k)
{
  for (int q = 0; q < k; q++)
  {
    wb_ctx *c = jobs[q];
    c->n_ambiguous = b->hOut->startAmb[q + 1] - b->hOut->startAmb[q];
    c->n_ground = b->hOut->ground[q];
    c->clsFinal = ((const ClsArgs *)c->clsArgs)->cls;
    c->clsStaged = false;
    c->clsHost = nullptr;
    c->stage = 3;
  }
}

/* One cloud: the fused sequence with one job, launched directly on the
 * context's stream (stage events between the passes), then the class bytes
 * copied out.  Synchronous. */
int wb_classify_impl(wb_ctx *c, const wb_params *p, uint8_t *cls, int onDevice)
{
  int rc = wb_classify_stage(c, p, cls, onDevice);
  if (rc)
    return rc;
  std::string err;
  if (!c->batch && (rc = wb_batch_create(c->device, &c->batch, err)))
    return wb_fail(c, rc, err);
  WbBatch *b = c->batch;
  int shape = clampShape(c->shape);
  if ((rc = fillTable(b, &c, 1, c->chunk, 0, err)))
    return wb_fail(c, rc, "wb_classify: " + err);
  unsigned grids[3];
  WB_CUDA(c, batchGrids(b, shape, grids));
  WB_CUDA(c, enqueueBatch(b, c->stream, shape, grids, c));
  c->launches += 9;
  ClsArgs *a = (ClsArgs *)c->clsArgs;
  if (!onDevice && c->n)
    WB_CUDA(c, cudaMemcpyAsync(cls, a->cls, c->n, cudaMemcpyDefault, c->stream));
  if (!onDevice && c->n && a->marginOut)
    WB_CUDA(c, cudaMemcpyAsync(c->marginDst, a->marginOut, c->n * 4, cudaMemcpyDefault, c->stream));
  wb_mark(c, "cls_download");
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  wb_batch_collect(b, &c, 1);
  return 0;
}

/* Search over the fused fast pass's settings on staged jobs, each setting
 * timed (best of two) on the whole of every job given: first every column
 * density with a group shape and a one-point shape, then the other shapes at
 * the best density, then the chunk sizes.  The jobs' grids are rebuilt for
 * each density and left with the chosen one.  Labels do not depend on any
 * of the settings. */
int wb_autotune_jobs(WbBatch *b, const WbTuneJob *jobs, int k, cudaStream_t s, int *shape, int *chunk,
                     double *gridPoints, std::string &err)
{
  int rc = 0;
  std::vector<wb_ctx *> ctxs(k);
  for (int q = 0; q < k; q++)
    ctxs[q] = jobs[q].c;
  auto timeIt = [&](int sh, int ch) -> float {   // best of two runs
    float best = 1e30f;
    for (int r = 0; r < 2; r++)
    {
      float ms = 0;
      if (rc == 0 && (rc = wb_batch_time(b, ctxs.data(), k, 0, sh, ch, s, &ms, err)) == 0)
        best = std::min(best, ms);
    }
    return best;
  };
  auto regrid = [&](double gp) -> bool {
    for (int q = 0; q < k && rc == 0; q++)
    {
      wb_ctx *c = jobs[q].c;
      if (c->grid_points == gp && c->clsStaged)
        continue;
      c->grid_points = gp;
      const double *g = c->grid_bounds;
      rc = wb_grid_impl(c, g[0], g[1], g[2], g[3]);
      if (rc == 0)
        rc = wb_classify_stage(c, jobs[q].p, jobs[q].cls, jobs[q].onDevice);
      if (rc == 0 && cudaStreamSynchronize(c->stream) != cudaSuccess)
        rc = WB_ECUDA;
      if (rc && err.empty())
        err = c->err;
    }
    return rc == 0;
  };
  const int ch0 = *chunk > 0 ? *chunk : 1;
  static const double kDensity[] = {32, 48, 64, 96};
  static const int kProbe[] = {0, 3};   // a column-group shape and a one-point shape
  float best = 1e30f;
  int bestShape = clampShape(*shape), bestChunk = ch0;
  double bestGp = *gridPoints > 0 ? *gridPoints : 64;
  bool warm = false;
  for (double gp : kDensity)
  {
    if (!regrid(gp))
      break;
    if (!warm)
    {
      timeIt(kProbe[0], ch0);
      warm = true;
    }
    for (int sh : kProbe)
    {
      float t = timeIt(sh, sh < 3 ? 1 : 4);
      if (t < best)
      {
        best = t;
        bestGp = gp;
        bestShape = sh;
        bestChunk = sh < 3 ? 1 : 4;
      }
    }
  }
  regrid(bestGp);
  const int probeChunk = bestChunk;
  for (int sh = 0; sh < WB_N_SHAPES; sh++)
  {
    if (sh == kProbe[0] || sh == kProbe[1])
      continue;
    float t = timeIt(sh, sh < 3 ? 1 : 4);
    if (t < best)
    {
      best = t;
      bestShape = sh;
      bestChunk = sh < 3 ? 1 : 4;
    }
  }
  (void)probeChunk;
  static const int kChunk[] = {1, 2, 4, 16};
  const int c0 = bestChunk;
  for (int ch : kChunk)
  {
    if (ch == c0)
      continue;
    float t = timeIt(bestShape, ch);
    if (t < best)
    {
      best = t;
      bestChunk = ch;
    }
  }
  if (rc)
    return rc;
  *shape = bestShape;
  *chunk = bestChunk;
  *gridPoints = bestGp;
  return 0;
}

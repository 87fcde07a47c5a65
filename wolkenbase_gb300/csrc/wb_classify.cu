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
 * One warp classifies one point.  It walks rings of grid columns outward from
 * the point, so directions from every side arrive early, and stops as soon as
 * the directions seen surround the point.  Per column it first checks whether
 * the column's lowest point could be inside the hyperboloid at the column's
 * nearest distance.  Each candidate is tested in FP32 in a frame centred on p
 * (integer record differences times the scale); the few whose FP32 value lies
 * within 1e-5 of the boundary, and points outside the octree root cube (which
 * the reference treats through their leaf's cube), are tested exactly in
 * FP64 as the reference computes it.  Directions are FP32 atan2 values in the
 * reference's integer angle unit; 64 bins keep each bin's extremes, and the
 * largest circular gap follows from them.  With the direction error bounded
 * by kMargin units, a gap estimate below 144 degrees - 2*kMargin proves
 * "surrounded" and one above 144 degrees + 2*kMargin proves the opposite;
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
#include "wb_internal.h"
#include "wb_device.cuh"
#include "angle_tables.h"

namespace
{
constexpr int kWarps = 4;
constexpr int kBins = 64;
constexpr uint32_t kStray = 0x80000000u;
/* bound on |FP32 direction - atan2i| in angle units (2^31 per turn); the
 * FP32 error is below 400 units, so this is a tenfold safety factor. */
constexpr uint32_t kMargin = 4096;

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
  const int32_t *owner;
  const TileRes *tiles;
  const double *tanT, *sinT, *cosT;
  uint8_t *label;
  /* grid */
  double gx0, gy0, cell;
  int nx, ny;
  uint64_t ncell;
  const uint32_t *cellStart;
  const int32_t *cellBox;
  const int32_t *gx, *gy, *gz;
  const uint32_t *gpos;
  int snx, sny;
  const int32_t *superBox;
  double zmin;
  int exactInts;   /* decode strictly increasing and 32-bit record differences exact */
  /* ambiguous points for the exact pass */
  uint32_t *ambList;
  uint32_t *ambCount;
  const uint32_t *work;   /* exact pass: store positions to classify */
  uint32_t nwork;
};

__device__ __forceinline__ double decA(const ClsArgs &a, int ax, int32_t q)
{
  return wb_decode(q, a.off[ax], a.scale[ax], a.unit);
}

struct Hyp
{
  double cx, cy, cz, por2;      /* exact Hyperboloid members (centre, polar radius^2) */
  double px, py;                /* the point, decoded                                  */
  int32_t qx, qy, qz;           /* the point, record integers                          */
  float sx, sy, sz;             /* metres per record unit                              */
  float czp, s2, por2f;         /* cz - pz, slope^2, por^2 in FP32                     */
};

/* OctStore::pointsIn membership of one candidate, exactly: Hyperboloid::in on
 * the decoded doubles; for a point outside the root cube, its leaf cube must
 * meet the hyperboloid (Octree::findBlocks) and then either all eight corners
 * are inside (the whole block is taken) or the point itself is. */
__device__ bool memberExact(const ClsArgs &a, const Hyp &h, uint32_t gp, int32_t qx, int32_t qy, int32_t qz)
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
__device__ __forceinline__ bool boxMeets(const Hyp &h, const int32_t *box, uint64_t N, uint64_t c)
{
  int32_t bx0 = box[c];
  if (bx0 == INT32_MAX)
    return false;   // empty block
  float xl = (float)(bx0 - h.qx) * h.sx, xh = (float)(box[3 * N + c] - h.qx) * h.sx;
  float yl = (float)(box[N + c] - h.qy) * h.sy, yh = (float)(box[4 * N + c] - h.qy) * h.sy;
  float zd = (float)(h.qz - box[2 * N + c]) * h.sz + h.czp;
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

template <bool EXACT>
__global__ void __launch_bounds__(32 * kWarps) classifyRings(ClsArgs a)
{
  __shared__ uint32_t bmin[kWarps][kBins], bmax[kWarps][kBins];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint64_t item = (uint64_t)blockIdx.x * kWarps + w;
  if (item >= (EXACT ? (uint64_t)a.nwork : a.nd))
    return;
  uint64_t j = EXACT ? a.work[item] : item;
  int32_t k = a.owner[j];
  if (k < 0)
  {
    if (lane == 0)
      a.label[j] = 0;
    return;
  }
  Hyp h;
  h.qx = a.sx[j];
  h.qy = a.sy[j];
  h.qz = a.sz[j];
  double hs = a.tiles[k].h;
  h.px = decA(a, 0, h.qx);
  h.py = decA(a, 1, h.qy);
  double pz = decA(a, 2, h.qz);
  // Hyperboloid(v, hs, slope), v = p - (0,0,thickness)  (shape.cpp:119-125)
  double por = hs * (a.slope * a.slope);
  h.por2 = por * por;
  h.cx = h.px + 0;
  h.cy = h.py + 0;
  h.cz = (pz - a.thickness) + por;
  h.sx = (float)(a.scale[0] * a.unit);
  h.sy = (float)(a.scale[1] * a.unit);
  h.sz = (float)(a.scale[2] * a.unit);
  h.czp = (float)(h.cz - pz);
  h.s2 = (float)(a.slope * a.slope);
  h.por2f = (float)h.por2;
  for (int b = lane; b < kBins; b += 32)
  {
    bmin[w][b] = 0xffffffffu;
    bmax[w][b] = 0;
  }
  __syncwarp();
  // horizontal reach of the hyperboloid at the lowest point of the cloud
  double zdMax = h.cz - a.zmin;
  double reach2 = (zdMax * zdMax - h.por2) / (a.slope * a.slope);
  double reach = reach2 > 0 ? sqrt(reach2) * (1 + 1e-6) + 1e-6 : 0.0;
  int ci = (int)floor((h.px - a.gx0) / a.cell), cj = (int)floor((h.py - a.gy0) / a.cell);
  int kmax = (int)ceil(reach / a.cell) + 1;
  bool surrounded = false, ambiguous = false;
  const bool fast = !EXACT && a.exactInts;
  // Adds the directions of column c's points that are inside; returns whether any was.
  auto column = [&](uint64_t cc) -> bool {
    bool got = false;
    uint32_t b = a.cellStart[cc], e = a.cellStart[cc + 1];
    for (uint32_t t = b + lane; t < e; t += 32)
    {
      int32_t qx = a.gx[t], qy = a.gy[t], qz = a.gz[t];
      uint32_t gp = a.gpos[t];
      uint32_t u;
      if (fast)
      {
        int32_t dxi = qx - h.qx, dyi = qy - h.qy;
        if (dxi == 0 && dyi == 0)
          continue;   // dist(p,q) == 0: no direction (classify.cpp:142,153)
        bool in;
        float dx = (float)dxi * h.sx, dy = (float)dyi * h.sy;
        if (gp & kStray)
          in = memberExact(a, h, gp, qx, qy, qz);
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
          else
            in = memberExact(a, h, gp, qx, qy, qz);
        }
        if (!in)
          continue;
        float th = atan2f(dy, dx);
        int d = __float2int_rn(th * 341782637.79f);   // 2^30 / pi
        u = (uint32_t)d & 0x7fffffffu;
      }
      else
      {
        double x = decA(a, 0, qx), y = decA(a, 1, qy);
        if (wb_hypot(h.px - x, h.py - y) == 0)
          continue;
        if (!memberExact(a, h, gp, qx, qy, qz))
          continue;
        int d = wb_atan2i(y - h.py, x - h.px, a.tanT, a.sinT, a.cosT, WB_ATAN_SCALE_HI, WB_ATAN_SCALE_LO);
        u = (uint32_t)d & 0x7fffffffu;
      }
      atomicMin(&bmin[w][u >> 25], u);
      atomicMax(&bmax[w][u >> 25], u);
      got = true;
    }
    return got;
  };
  auto decide = [&]() {
    __syncwarp();
    int nocc;
    uint32_t gap = largestGap(bmin[w], bmax[w], lane, nocc);
    if (nocc >= 2)
      surrounded = (EXACT || !fast) ? gap < (uint32_t)WB_DEG144 : gap + 2 * kMargin < (uint32_t)WB_DEG144;
  };
  // Near field: rings of single columns around the point's column.
  const int kNear = 2;
  for (int ring = 0; ring <= kNear && ring <= kmax && !surrounded; ring++)
  {
    if (ci + ring < 0 || ci - ring >= a.nx || cj + ring < 0 || cj - ring >= a.ny)
      continue;
    int ncells = ring == 0 ? 1 : 8 * ring;
    bool gotAny = false;
    for (int m0 = 0; m0 < ncells; m0 += 32)
    {
      int m = m0 + lane;
      uint64_t c = 0;
      bool ok = false;
      if (m < ncells)
      {
        int di, dj;
        ringCell(ring, m, di, dj);
        int i = ci + di, jj = cj + dj;
        if (i >= 0 && i < a.nx && jj >= 0 && jj < a.ny)
        {
          c = (uint64_t)jj * a.nx + i;
          ok = a.cellStart[c] != a.cellStart[c + 1] && boxMeets(h, a.cellBox, a.ncell, c);
        }
      }
      unsigned mask = __ballot_sync(0xffffffffu, ok);
      while (mask)
      {
        int src = __ffs(mask) - 1;
        mask &= mask - 1;
        gotAny |= column(__shfl_sync(0xffffffffu, c, src));
      }
    }
    if (__any_sync(0xffffffffu, gotAny))
      decide();
  }
  // Far field: rings of super-cells (WB_SUPER x WB_SUPER columns) pruned as a
  // block; columns already visited in the near field are skipped.
  const int S = WB_SUPER;
  int si = ci >= 0 ? ci / S : -((-ci + S - 1) / S), sj = cj >= 0 ? cj / S : -((-cj + S - 1) / S);
  int smax = (int)ceil(reach / (S * a.cell)) + 1;
  const uint64_t NS = (uint64_t)a.snx * a.sny;
  for (int sr = 0; sr <= smax && !surrounded && kmax > kNear; sr++)
  {
    if (si + sr < 0 || si - sr >= a.snx || sj + sr < 0 || sj - sr >= a.sny)
      continue;
    int nsc = sr == 0 ? 1 : 8 * sr;
    bool gotAny = false;
    for (int m0 = 0; m0 < nsc; m0 += 32)
    {
      int m = m0 + lane;
      int SI = 0, SJ = 0;
      bool ok = false;
      if (m < nsc)
      {
        int di, dj;
        ringCell(sr, m, di, dj);
        SI = si + di;
        SJ = sj + dj;
        if (SI >= 0 && SI < a.snx && SJ >= 0 && SJ < a.sny)
          ok = boxMeets(h, a.superBox, NS, (uint64_t)SJ * a.snx + SI);
      }
      unsigned mask = __ballot_sync(0xffffffffu, ok);
      while (mask)
      {
        int src = __ffs(mask) - 1;
        mask &= mask - 1;
        int bi = __shfl_sync(0xffffffffu, SI, src) * S, bj = __shfl_sync(0xffffffffu, SJ, src) * S;
        // lanes 0..S*S-1 take the block's columns
        uint64_t c = 0;
        bool cok = false;
        if (lane < S * S)
        {
          int i = bi + lane % S, jj = bj + lane / S;
          int cheb = max(abs(i - ci), abs(jj - cj));
          if (i < a.nx && jj < a.ny && cheb > kNear)
          {
            c = (uint64_t)jj * a.nx + i;
            cok = a.cellStart[c] != a.cellStart[c + 1] && boxMeets(h, a.cellBox, a.ncell, c);
          }
        }
        unsigned cm = __ballot_sync(0xffffffffu, cok);
        while (cm)
        {
          int cs = __ffs(cm) - 1;
          cm &= cm - 1;
          gotAny |= column(__shfl_sync(0xffffffffu, c, cs));
        }
      }
    }
    if (__any_sync(0xffffffffu, gotAny))
      decide();
  }
  if (!surrounded && fast)
  {
    int nocc;
    __syncwarp();
    uint32_t gap = largestGap(bmin[w], bmax[w], lane, nocc);
    ambiguous = nocc >= 2 && gap < (uint32_t)WB_DEG144 + 2 * kMargin;
  }
  if (lane == 0)
  {
    a.label[j] = surrounded ? 1 : 2;
    if (ambiguous)
      a.ambList[atomicAdd(a.ambCount, 1u)] = (uint32_t)j;
  }
}

__global__ void scatterCls(uint64_t n, const uint32_t *__restrict__ storeOf, const int32_t *__restrict__ owner,
                           const uint8_t *__restrict__ label, uint8_t *__restrict__ cls)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t j = storeOf[i];
    if (owner[j] >= 0)
      cls[i] = label[j];
  }
}

__global__ void groundCount(uint64_t nd, const int32_t *__restrict__ owner, const uint8_t *__restrict__ label,
                            TileRes *__restrict__ tiles)
{
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nd; j += (uint64_t)gridDim.x * blockDim.x)
    if (owner[j] >= 0 && label[j] == 2)
      atomicAdd(&tiles[owner[j]].nGround, 1);
}

__global__ void zeroGround(uint64_t T, TileRes *__restrict__ tiles)
{
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < T; k += (uint64_t)gridDim.x * blockDim.x)
    tiles[k].nGround = 0;
}
}  // namespace

/* Decoding is strictly increasing in every record integer when the step
 * scale*unit is at least four ulps of every coordinate the root cube spans;
 * then equal decoded doubles mean equal integers, and FP32 differences of
 * integers stand for differences of the doubles. */
static bool decodeIsExact(const WbGeom &g, const double mn[3], const double mx[3])
{
  for (int a = 0; a < 3; a++)
  {
    double step = fabs(g.scale[a] * g.unit);
    double mag = fmax(fabs(mn[a]), fabs(mx[a])) + fabs(g.off[a] * g.unit) + step;
    if (!(step > 0) || step < 4 * ldexp(mag, -52))
      return false;
  }
  return true;
}

int wb_classify_impl(wb_ctx *c, const wb_params *p, uint8_t *cls, int onDevice)
{
  if (c->stage < 2)
    return wb_fail(c, WB_ESTATE, "wb_classify: scan the tiles first");
  if (!cls && c->n)
    return wb_fail(c, WB_EINVAL, "wb_classify: cls must not be NULL");
  if (!(p->max_slope > 0))
    return wb_fail(c, WB_EINVAL, "wb_classify: max_slope must be > 0");
  int rc;
  uint64_t nd = c->nd, n = c->n;
  if ((rc = wb_ensure(c, c->label, nd + 64)) || (rc = wb_ensure(c, c->angleT, (511 + 512 + 512) * 8)) ||
      (rc = wb_ensure(c, c->ambiguous, nd * 4 + 64)))
    return rc;
  if (!onDevice && (rc = wb_ensure(c, c->clsDev, n + 64)))
    return rc;
  double *tab = (double *)c->angleT.p;
  WB_CUDA(c, cudaMemcpyAsync(tab, kWbTan, 511 * 8, cudaMemcpyHostToDevice, c->stream));
  WB_CUDA(c, cudaMemcpyAsync(tab + 511, kWbSin, 512 * 8, cudaMemcpyHostToDevice, c->stream));
  WB_CUDA(c, cudaMemcpyAsync(tab + 1023, kWbCos, 512 * 8, cudaMemcpyHostToDevice, c->stream));
  uint8_t *clsDev = onDevice ? cls : (uint8_t *)c->clsDev.p;
  if (!onDevice && n)
    WB_CUDA(c, cudaMemcpyAsync(clsDev, cls, n, cudaMemcpyHostToDevice, c->stream));
  wb_mark(c, "cls_upload");
  ClsArgs a;
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
  a.owner = (const int32_t *)c->owner.p;
  a.tiles = (const TileRes *)c->tileRes.p;
  a.tanT = tab;
  a.sinT = tab + 511;
  a.cosT = tab + 1023;
  a.label = (uint8_t *)c->label.p;
  a.gx0 = c->grid.x0;
  a.gy0 = c->grid.y0;
  a.cell = c->grid.cell;
  a.nx = c->grid.nx;
  a.ny = c->grid.ny;
  a.ncell = c->grid.ncell;
  a.cellStart = (const uint32_t *)c->cellStart.p;
  a.cellBox = (const int32_t *)c->cellBox.p;
  a.gx = (const int32_t *)c->gx.p;
  a.gy = (const int32_t *)c->gy.p;
  a.gz = (const int32_t *)c->gz.p;
  a.gpos = (const uint32_t *)c->gpos.p;
  a.snx = c->grid.snx;
  a.sny = c->grid.sny;
  a.superBox = (const int32_t *)c->superBox.p;
  a.zmin = (g.off[2] + g.scale[2] * (double)c->grid.zminInt) * g.unit;
  bool fits32 = true;
  for (int k = 0; k < 3; k++)
    fits32 = fits32 && (int64_t)c->grid.imax[k] - (int64_t)c->grid.imin[k] < ((int64_t)1 << 30);
  a.exactInts = (decodeIsExact(g, mn, mx) && fits32) ? 1 : 0;
  a.ambList = (uint32_t *)c->ambiguous.p;
  a.ambCount = (uint32_t *)((char *)c->small.p + 448);
  a.work = nullptr;
  a.nwork = 0;
  WB_CUDA(c, cudaMemsetAsync(a.ambCount, 0, 4, c->stream));
  if (nd)
  {
    { classifyRings<false><<<(unsigned)((nd + kWarps - 1) / kWarps), 32 * kWarps, 0, c->stream>>>(a); ++c->launches; }
    WB_CUDA(c, cudaGetLastError());
  }
  wb_mark(c, "classify");
  uint32_t namb = 0;
  WB_CUDA(c, cudaMemcpyAsync(&namb, a.ambCount, 4, cudaMemcpyDeviceToHost, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  c->n_ambiguous = namb;
  if (namb)
  {
    a.work = a.ambList;
    a.nwork = namb;
    { classifyRings<true><<<(namb + kWarps - 1) / kWarps, 32 * kWarps, 0, c->stream>>>(a); ++c->launches; }
    WB_CUDA(c, cudaGetLastError());
  }
  wb_mark(c, "classify_exact");
  unsigned gsz = (unsigned)std::min<uint64_t>((n + 255) / 256 + 1, (uint64_t)c->sm_count * 16);
  { zeroGround<<<gsz, 256, 0, c->stream>>>(c->n_tiles, (TileRes *)c->tileRes.p); ++c->launches; }
  { groundCount<<<gsz, 256, 0, c->stream>>>(nd, a.owner, a.label, (TileRes *)c->tileRes.p); ++c->launches; }
  if (n)
    { scatterCls<<<gsz, 256, 0, c->stream>>>(n, (const uint32_t *)c->storeOf.p, a.owner, a.label, clsDev); ++c->launches; }
  if (!onDevice && n)
    WB_CUDA(c, cudaMemcpyAsync(cls, clsDev, n, cudaMemcpyDeviceToHost, c->stream));
  WB_CUDA(c, cudaGetLastError());
  wb_mark(c, "cls_download");
  c->stage = 3;
  return 0;
}

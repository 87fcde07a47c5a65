/* classifyCylinder on the GPU (classify.cpp:96-173).
 *
 * The reference classifies point p by growing a std::set of integer
 * directions dir(p,q) to the points q inside the downward hyperboloid
 * Hyperboloid(p - (0,0,thickness), tile.hyperboloidSize, maxSlope), stopping
 * as soon as no circular gap between successive directions reaches 144
 * degrees (surround, classify.cpp:67-94).  Adding directions can only shrink
 * gaps and the pruning it does never opens one, so the label is a function of
 * the whole neighbour set: 1 (not ground) if it surrounds p, else 2.
 *
 * Here one warp classifies one point: it walks the node hierarchy depth-first,
 * pruning boxes the hyperboloid cannot reach, tests the points of each leaf
 * it reaches (32 lanes at a time), and keeps, for 64 direction bins of 2^25
 * units, the smallest and largest direction seen.  Gaps inside a bin are
 * shorter than 144 degrees, so the largest circular gap of the whole set is
 * the largest gap between the last direction of one occupied bin and the first
 * of the next one: the test is exact.  The warp stops when that gap drops
 * below 144 degrees.  A point is classified with the hyperboloid size of its
 * owner tile, the last tile in flowsnake order whose cylinder contains it,
 * because that tile's classification is the one the reference keeps.
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
constexpr int kStack = 192;
constexpr int kBins = 64;

struct ClsArgs
{
  uint64_t nd;
  double off[3], scale[3], unit;
  double slope, thickness;
  const int32_t *child, *nodeBox, *leafBox;
  uint64_t N, L;
  const uint32_t *leafFirst, *leafCount;
  const uint64_t *leafKey;
  const uint8_t *leafLev;
  double rootLo[3], rootSide;
  const int32_t *sx, *sy, *sz;
  const int32_t *owner;
  const TileRes *tiles;
  const double *tanT, *sinT, *cosT;
  uint8_t *label;
};

__device__ __forceinline__ double decA(const ClsArgs &a, int ax, int32_t q)
{
  return wb_decode(q, a.off[ax], a.scale[ax], a.unit);
}

/* Could any point of the box lie inside the hyperboloid?  The most favourable
 * point of a box is its lowest corner height at the xy position nearest the
 * axis; a small relative slack keeps this conservative. */
__device__ __forceinline__ bool boxMeetsHyp(const ClsArgs &a, const int32_t *box, uint64_t stride, uint64_t id,
                                            double cx, double cy, double cz, double por2)
{
  double x0 = decA(a, 0, box[0 * stride + id]), x1 = decA(a, 0, box[3 * stride + id]);
  double y0 = decA(a, 1, box[1 * stride + id]), y1 = decA(a, 1, box[4 * stride + id]);
  double z0 = decA(a, 2, box[2 * stride + id]);
  double dx = cx < x0 ? x0 - cx : (cx > x1 ? cx - x1 : 0.0);
  double dy = cy < y0 ? y0 - cy : (cy > y1 ? cy - y1 : 0.0);
  double zd = cz - z0;
  if (!(zd > 0))
    return false;
  double lhs = zd * zd - a.slope * a.slope * (dx * dx + dy * dy);
  return lhs >= por2 - 1e-9 * (zd * zd + por2) - 1e-12;
}

__global__ void __launch_bounds__(32 * kWarps) classifyKernel(ClsArgs a)
{
  __shared__ int32_t stack[kWarps][kStack];
  __shared__ uint32_t bmin[kWarps][kBins], bmax[kWarps][kBins];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint64_t j = (uint64_t)blockIdx.x * kWarps + w;
  if (j >= a.nd)
    return;
  int32_t k = a.owner[j];
  if (k < 0)
  {
    if (lane == 0)
      a.label[j] = 0;
    return;
  }
  double h = a.tiles[k].h;
  double px = decA(a, 0, a.sx[j]), py = decA(a, 1, a.sy[j]), pz = decA(a, 2, a.sz[j]);
  // Hyperboloid(v, h, slope) with v = p - (0,0,thickness)  (shape.cpp:119-125)
  double por = h * (a.slope * a.slope);
  double por2 = por * por;
  double cx = px + 0, cy = py + 0, cz = (pz - a.thickness) + por;
  for (int b = lane; b < kBins; b += 32)
  {
    bmin[w][b] = 0xffffffffu;
    bmax[w][b] = 0;
  }
  __syncwarp();
  bool surrounded = false;
  int sp = 1;
  if (lane == 0)
    stack[w][0] = 0;
  __syncwarp();
  if (a.N == 0)
    sp = 0;
  while (sp > 0 && !surrounded)
  {
    int32_t code = stack[w][sp - 1];
    sp--;
    __syncwarp();
    if (code >= 0)
    {
      int32_t ch = -1;
      bool meet = false;
      if (lane < 8)
      {
        ch = a.child[(uint64_t)code * 8 + lane];
        if (ch >= 0)
          meet = boxMeetsHyp(a, a.nodeBox, a.N, (uint64_t)ch, cx, cy, cz, por2);
        else if (ch <= -2)
          meet = boxMeetsHyp(a, a.leafBox, a.L, (uint64_t)(-2 - ch), cx, cy, cz, por2);
      }
      unsigned m = __ballot_sync(0xffffffffu, meet);
      if (meet)
        stack[w][sp + __popc(m >> (lane + 1))] = ch;
      sp += __popc(m);
      __syncwarp();
      continue;
    }
    uint64_t l = (uint64_t)(-2 - code);
    uint32_t f = a.leafFirst[l], cnt = a.leafCount[l];
    // OctStore::pointsIn (octree.cpp:1214-1242): a block counts only if its
    // cube meets the shape (Octree::findBlocks); if all eight corners are
    // inside, all its points are taken without testing them one by one.
    // The two differ from testing every point only for points outside the
    // root cube (Octree::sizeFit can leave a sliver of the cloud below it).
    bool cubeTest = false;
    {
      double lx, ly, lz, ls;
      wb_leaf_cube(a.leafKey[l], a.leafLev[l], a.rootLo, a.rootSide, lx, ly, lz, ls);
      if (lane == 0)
        cubeTest = wb_hyp_in(cx, cy, cz, por2, a.slope, wb_clamp_toward(cx, lx, ls), wb_clamp_toward(cy, ly, ls),
                             lz - ls / 2);
      else if (lane <= 8)
      {
        int n = lane - 1;
        cubeTest = wb_hyp_in(cx, cy, cz, por2, a.slope, (n & 1) ? lx + ls / 2 : lx - ls / 2,
                             (n & 2) ? ly + ls / 2 : ly - ls / 2, (n & 4) ? lz + ls / 2 : lz - ls / 2);
      }
    }
    unsigned cb = __ballot_sync(0xffffffffu, cubeTest);
    if (!(cb & 1))
      continue;
    const bool allIn = (cb & 0x1feu) == 0x1feu;
    for (uint32_t t0 = 0; t0 < cnt; t0 += 32)
    {
      uint32_t t = t0 + lane;
      if (t < cnt)
      {
        uint32_t q = f + t;
        double qx = decA(a, 0, a.sx[q]), qy = decA(a, 1, a.sy[q]), qz = decA(a, 2, a.sz[q]);
        if (allIn || wb_hyp_in(cx, cy, cz, por2, a.slope, qx, qy, qz))
        {
          double dx = qx - px, dy = qy - py;
          if (wb_hypot(px - qx, py - qy) != 0)
          {
            int d = wb_atan2i(dy, dx, a.tanT, a.sinT, a.cosT, WB_ATAN_SCALE_HI, WB_ATAN_SCALE_LO);
            uint32_t u = (uint32_t)d & 0x7fffffffu;
            atomicMin(&bmin[w][u >> 25], u);
            atomicMax(&bmax[w][u >> 25], u);
          }
        }
      }
    }
    __syncwarp();
    // exact largest circular gap from the bin extremes
    uint32_t mn0 = bmin[w][lane], mn1 = bmin[w][lane + 32];
    uint32_t mx0 = bmax[w][lane], mx1 = bmax[w][lane + 32];
    unsigned occLo = __ballot_sync(0xffffffffu, mn0 != 0xffffffffu);
    unsigned occHi = __ballot_sync(0xffffffffu, mn1 != 0xffffffffu);
    uint64_t occ = ((uint64_t)occHi << 32) | occLo;
    int nocc = __popcll(occ);
    bool sur = false;
    if (nocc >= 2)
    {
      uint32_t worst = 0;
      for (int half = 0; half < 2; half++)
      {
        int b = lane + 32 * half;
        if ((occ >> b) & 1)
        {
          // next occupied bin after b, circularly
          uint64_t rot = (b == 63) ? 0 : (occ >> (b + 1));
          int nb = rot ? b + 1 + __ffsll((long long)rot) - 1 : __ffsll((long long)occ) - 1;
          uint32_t gap = (bmin[w][nb] - (half ? mx1 : mx0)) & 0x7fffffffu;
          worst = max(worst, gap);
        }
      }
      for (int o = 16; o; o >>= 1)
        worst = max(worst, __shfl_xor_sync(0xffffffffu, worst, o));
      sur = worst < (uint32_t)WB_DEG144;
    }
    else if (nocc == 1)
    {
      // one bin: at least two distinct directions and every gap < 144 degrees is impossible
      sur = false;
    }
    surrounded = sur;
  }
  if (lane == 0)
    a.label[j] = surrounded ? 1 : 2;
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

int wb_classify_impl(wb_ctx *c, const wb_params *p, uint8_t *cls, int onDevice)
{
  if (c->stage < 2)
    return wb_fail(c, WB_ESTATE, "wb_classify: scan the tiles first");
  if (!cls && c->n)
    return wb_fail(c, WB_EINVAL, "wb_classify: cls must not be NULL");
  int rc;
  uint64_t nd = c->nd, n = c->n;
  if ((rc = wb_ensure(c, c->label, nd + 64)) || (rc = wb_ensure(c, c->angleT, (511 + 512 + 512) * 8)))
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
  for (int k = 0; k < 3; k++)
  {
    a.off[k] = c->g.off[k];
    a.scale[k] = c->g.scale[k];
  }
  a.unit = c->g.unit;
  a.slope = p->max_slope;
  a.thickness = p->thickness;
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
    a.rootLo[k] = c->g.root_lo[k];
  a.rootSide = c->g.root_side;
  a.sx = (const int32_t *)c->sx.p;
  a.sy = (const int32_t *)c->sy.p;
  a.sz = (const int32_t *)c->sz.p;
  a.owner = (const int32_t *)c->owner.p;
  a.tiles = (const TileRes *)c->tileRes.p;
  a.tanT = tab;
  a.sinT = tab + 511;
  a.cosT = tab + 1023;
  a.label = (uint8_t *)c->label.p;
  if (nd)
  {
    { classifyKernel<<<(unsigned)((nd + kWarps - 1) / kWarps), 32 * kWarps, 0, c->stream>>>(a); ++c->launches; }
    WB_CUDA(c, cudaGetLastError());
  }
  wb_mark(c, "classify");
  unsigned g = (unsigned)std::min<uint64_t>((n + 255) / 256 + 1, (uint64_t)c->sm_count * 16);
  { zeroGround<<<g, 256, 0, c->stream>>>(c->n_tiles, (TileRes *)c->tileRes.p); ++c->launches; }
  { groundCount<<<g, 256, 0, c->stream>>>(nd, a.owner, a.label, (TileRes *)c->tileRes.p); ++c->launches; }
  if (n)
    { scatterCls<<<g, 256, 0, c->stream>>>(n, (const uint32_t *)c->storeOf.p, a.owner, a.label, clsDev); ++c->launches; }
  if (!onDevice && n)
    WB_CUDA(c, cudaMemcpyAsync(cls, clsDev, n, cudaMemcpyDeviceToHost, c->stream));
  WB_CUDA(c, cudaGetLastError());
  wb_mark(c, "cls_download");
  c->stage = 3;
  return 0;
}

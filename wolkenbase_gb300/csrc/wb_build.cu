/* Octree build on the GPU: the replacement for OctStore::put / split.
 *
 * The reference inserts points one at a time and splits a block when a 538th
 * distinct point arrives (octree.cpp:620-662, 1295-1338).  Because a split
 * never merges and de-duplication is by exact xyz, the final tree depends only
 * on the set of distinct points: a node is internal iff its cube holds more
 * than 537 distinct points (the root is always internal), and every non-empty
 * octant of an internal node that is not itself internal is a leaf block.
 * The build therefore needs no insertion order:
 *
 *   K1  decode X,Y,Z like las.cpp:808 and compute a 63-bit Morton key whose
 *       every bit is one of the reference's x>=center decisions
 *   K2  stable radix sort of (key, input index)
 *   K3  mark duplicates (same doubles; the last one read survives, as
 *       OctBuffer::put overwrites) and compact
 *   K4  common-prefix level of keys 537 apart; the leaf level of a point is
 *       1 + the largest such level over the 538-point windows that contain it
 *       (a node holds >537 points iff one window fits inside it)
 *   K5  leaf starts, leaf table, per-leaf order by input index, leaf boxes
 *   K6  explicit node hierarchy (8 children per internal node) with boxes,
 *       used by the cylinder and hyperboloid queries
 */
#include <cuda_runtime.h>
#include <cstdint>
#include <cstring>
#include <cmath>
#include "wb_internal.h"
#include "wb_device.cuh"

namespace
{
constexpr int kWindow = WB_RECORDS + 1;   // 538 points: the first that forces a split

struct KeyArgs
{
  const uint8_t *rec;
  uint64_t n;
  uint32_t stride;
  double off[3], scale[3], unit;
  double lo[3], cell;
  /* Fixed-point form of the level-21 cell coordinate, per axis:
     t(X) = (C + (X - x0) * R) / 2^shift, with |X - x0| <= dmax.  A point
     whose fraction lies more than eps from an integer takes floor(t); the
     rest (and all of an axis with fixed = 0) take the exact FP64 path. */
  int fixed[3], shift[3];
  long long x0[3], dmax[3], rfix[3], cfix[3], eps[3];
};

__device__ __forceinline__ void loadXYZ(const uint8_t *rec, uint32_t stride, uint64_t i, int32_t &x, int32_t &y,
                                        int32_t &z)
{
  const uint8_t *p = rec + i * (uint64_t)stride;
  if ((stride & 3) == 0)
  {
    const int32_t *q = (const int32_t *)p;
    x = q[0];
    y = q[1];
    z = q[2];
  }
  else
  {
    int32_t v[3];
    memcpy(v, p, 12);
    x = v[0];
    y = v[1];
    z = v[2];
  }
}

__global__ void keyKernel(KeyArgs a, uint64_t *__restrict__ keys, uint32_t *__restrict__ idx)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    int32_t q[3];
    loadXYZ(a.rec, a.stride, i, q[0], q[1], q[2]);
    uint32_t k[3];
#pragma unroll
    for (int ax = 0; ax < 3; ax++)
    {
      const long long d = (long long)q[ax] - a.x0[ax];
      bool done = false;
      if (a.fixed[ax] && d >= -a.dmax[ax] && d <= a.dmax[ax])
      {
        const long long tf = d * a.rfix[ax] + a.cfix[ax];
        const long long k0 = tf >> a.shift[ax];
        const long long fr = tf - k0 * (1ll << a.shift[ax]);
        if (fr > a.eps[ax] && fr < (1ll << a.shift[ax]) - a.eps[ax])
        {
          const long long kMax = (1 << WB_LEVELS) - 1;
          k[ax] = (uint32_t)(k0 < 0 ? 0 : (k0 > kMax ? kMax : k0));
          done = true;
        }
      }
      if (!done)
        k[ax] = wb_cell_index(wb_decode(q[ax], a.off[ax], a.scale[ax], a.unit), a.lo[ax], a.cell);
    }
    keys[i] = wb_morton(k[0], k[1], k[2]);
    idx[i] = (uint32_t)i;
  }
}

__device__ __forceinline__ bool sameDoubles(const KeyArgs &a, uint32_t i, uint32_t j)
{
  int32_t p[3], q[3];
  loadXYZ(a.rec, a.stride, i, p[0], p[1], p[2]);
  loadXYZ(a.rec, a.stride, j, q[0], q[1], q[2]);
#pragma unroll
  for (int ax = 0; ax < 3; ax++)
    if (wb_decode(p[ax], a.off[ax], a.scale[ax], a.unit) != wb_decode(q[ax], a.off[ax], a.scale[ax], a.unit))
      return false;
  return true;
}

/* survivor[i] = 1 unless a later record in the same key run has the same xyz. */
__global__ void survivorKernel(KeyArgs a, const uint64_t *__restrict__ keys, const uint32_t *__restrict__ idx,
                               uint32_t *__restrict__ surv)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t s = 1;
    uint64_t k = keys[i];
    for (uint64_t j = i + 1; j < a.n && keys[j] == k; j++)
      if (sameDoubles(a, idx[i], idx[j]))
      {
        s = 0;
        break;
      }
    surv[i] = s;
  }
}

__global__ void compactKernel(uint64_t n, const uint64_t *__restrict__ keys, const uint32_t *__restrict__ idx,
                              const uint32_t *__restrict__ surv, const uint32_t *__restrict__ rank,
                              uint64_t *__restrict__ dkey, uint32_t *__restrict__ didx)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    if (surv[i])
    {
      dkey[rank[i]] = keys[i];
      didx[rank[i]] = idx[i];
    }
}

/* cpl[s] = common levels of dkey[s] and dkey[s+537], s in [0, nd-538]. */
__global__ void cplKernel(const uint64_t *__restrict__ dkey, uint64_t nw, uint8_t *__restrict__ cpl)
{
  for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nw; s += (uint64_t)gridDim.x * blockDim.x)
    cpl[s] = (uint8_t)wb_common_levels(dkey[s], dkey[s + kWindow - 1]);
}

/* Prefix and suffix maxima inside aligned segments of kWindow windows
 * (van Herk / Gil-Werman): one warp per segment. */
__global__ void segMaxKernel(const uint8_t *__restrict__ cpl, uint64_t nw, uint8_t *__restrict__ pre,
                             uint8_t *__restrict__ suf)
{
  uint64_t seg = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  uint64_t b = seg * kWindow;
  if (b >= nw)
    return;
  uint64_t e = b + kWindow < nw ? b + kWindow : nw;
  int run = 0;
  for (uint64_t s0 = b; s0 < e; s0 += 32)
  {
    uint64_t s = s0 + lane;
    int v = s < e ? cpl[s] : 0;
    for (int o = 1; o < 32; o <<= 1)
    {
      int t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o)
        v = max(v, t);
    }
    v = max(v, run);
    if (s < e)
      pre[s] = (uint8_t)v;
    run = __shfl_sync(0xffffffffu, v, 31);
  }
  run = 0;
  uint64_t len = e - b;
  for (uint64_t r0 = 0; r0 < len; r0 += 32)
  {
    uint64_t r = r0 + lane;   // distance from the end
    uint64_t s = e - 1 - r;
    int v = r < len ? cpl[s] : 0;
    for (int o = 1; o < 32; o <<= 1)
    {
      int t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o)
        v = max(v, t);
    }
    v = max(v, run);
    if (r < len)
      suf[s] = (uint8_t)v;
    run = __shfl_sync(0xffffffffu, v, 31);
  }
}

/* lev[i] = 1 + max cpl over windows [s, s+537] containing i. */
__global__ void levelKernel(uint64_t nd, uint64_t nw, const uint8_t *__restrict__ pre, const uint8_t *__restrict__ suf,
                            uint8_t *__restrict__ lev, int *__restrict__ err)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += (uint64_t)gridDim.x * blockDim.x)
  {
    int d = 0;
    if (nw > 0)
    {
      uint64_t a = i >= (uint64_t)(kWindow - 1) ? i - (kWindow - 1) : 0;
      uint64_t b = i < nw - 1 ? i : nw - 1;
      if (a <= b)
      {
        uint64_t sa = a / kWindow, sb = b / kWindow;
        if (sa != sb)
          d = max((int)suf[a], (int)pre[b]);
        else if (a == sa * kWindow)
          d = pre[b];
        else
          d = suf[a];
      }
    }
    if (d >= WB_LEVELS)
    {
      atomicExch(err, 1);
      d = WB_LEVELS - 1;
    }
    lev[i] = (uint8_t)(d + 1);
  }
}

__device__ __forceinline__ uint64_t prefixAt(uint64_t key, int level)
{
  return level <= 0 ? 0 : key >> (63 - 3 * level);
}

__global__ void leafStartKernel(uint64_t nd, const uint64_t *__restrict__ dkey, const uint8_t *__restrict__ lev,
                                uint32_t *__restrict__ start)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t s = 1;
    if (i > 0)
    {
      int l = lev[i];
      s = (lev[i - 1] != l) || (prefixAt(dkey[i - 1], l) != prefixAt(dkey[i], l));
    }
    start[i] = s;
  }
}

__global__ void leafTableKernel(uint64_t nd, const uint64_t *__restrict__ dkey, const uint8_t *__restrict__ lev,
                                const uint32_t *__restrict__ start, const uint32_t *__restrict__ ex,
                                uint32_t *__restrict__ leafId, uint32_t *__restrict__ first,
                                uint8_t *__restrict__ leafLev, uint64_t *__restrict__ leafKey)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint32_t l = ex[i] + start[i] - 1;
    leafId[i] = l;
    if (start[i])
    {
      int lv = lev[i];
      first[l] = (uint32_t)i;
      leafLev[l] = (uint8_t)lv;
      uint64_t mask = (lv >= WB_LEVELS) ? ~0ULL : ~((1ULL << (63 - 3 * lv)) - 1);
      leafKey[l] = dkey[i] & mask;
    }
  }
}

__global__ void leafCountKernel(uint64_t L, uint64_t nd, const uint32_t *__restrict__ first, uint32_t *__restrict__ count)
{
  for (uint64_t l = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; l < L; l += (uint64_t)gridDim.x * blockDim.x)
    count[l] = (uint32_t)((l + 1 < L ? first[l + 1] : nd) - first[l]);
}

/* One block per leaf: bitonic sort of the leaf's input indices (<= 537, padded
 * to a power of two, at most 1024), gather of X/Y/Z into store order, integer
 * bounding box, and each stored record's store slot and leaf.  Each thread is
 * one comparator of a stage (kLeafThreads comparators per pass).  A stage
 * whose partners lie at most 32 apart touches only its warp's own 64-element
 * window, so between two such stages a warp barrier is enough. */
constexpr int kLeafThreads = 256;
__global__ void __launch_bounds__(kLeafThreads) leafSortKernel(KeyArgs a, const uint32_t *__restrict__ first,
                                                               const uint32_t *__restrict__ count,
                                                               const uint32_t *__restrict__ didx,
                                                               uint32_t *__restrict__ sidx, int32_t *__restrict__ sx,
                                                               int32_t *__restrict__ sy, int32_t *__restrict__ sz,
                                                               int32_t *__restrict__ box, uint32_t *__restrict__ storeOf,
                                                               uint64_t L,
                                                               double *__restrict__ xyzd, uint64_t nd)
{
  __shared__ uint32_t v[1024];
  __shared__ int32_t red[6][kLeafThreads / 32];
  const uint64_t l = blockIdx.x;
  if (l >= L)
    return;
  const uint32_t f = first[l], cnt = count[l];
  int P = 64;
  while (P < (int)cnt)
    P <<= 1;
  for (int t = threadIdx.x; t < P; t += kLeafThreads)
    v[t] = t < (int)cnt ? didx[f + t] : 0xffffffffu;
  __syncthreads();
  const int half = P >> 1;
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1)
    {
      // comparator t's lower element: (t / j) * 2j + t % j, with shifts (j is a power of two)
      const int lj = __ffs(j) - 1;
      for (int t = threadIdx.x; t < half; t += kLeafThreads)
      {
        const int i = ((t >> lj) << (lj + 1)) | (t & (j - 1)), u = i + j;
        const bool up = (i & k) == 0;
        const uint32_t x = v[i], y = v[u];
        if ((x > y) == up)
        {
          v[i] = y;
          v[u] = x;
        }
      }
      // a warp barrier suffices when this stage and the next both stay in
      // the warps' own 64-element windows
      const int jNext = j > 1 ? j >> 1 : k;
      if (j <= 32 && jNext <= 32 && half <= kLeafThreads)
        __syncwarp();
      else
        __syncthreads();
    }
  __syncthreads();
  int32_t mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
  for (int t = threadIdx.x; t < (int)cnt; t += kLeafThreads)
  {
    const uint32_t id = v[t];
    int32_t q[3];
    loadXYZ(a.rec, a.stride, id, q[0], q[1], q[2]);
    sidx[f + t] = id;
    sx[f + t] = q[0];
    sy[f + t] = q[1];
    sz[f + t] = q[2];
#pragma unroll
    for (int ax = 0; ax < 3; ax++)
      xyzd[(uint64_t)ax * nd + f + t] = wb_decode(q[ax], a.off[ax], a.scale[ax], a.unit);
    storeOf[id] = f + t;
#pragma unroll
    for (int ax = 0; ax < 3; ax++)
    {
      mn[ax] = min(mn[ax], q[ax]);
      mx[ax] = max(mx[ax], q[ax]);
    }
  }
#pragma unroll
  for (int ax = 0; ax < 3; ax++)
    for (int o = 16; o; o >>= 1)
    {
      mn[ax] = min(mn[ax], __shfl_xor_sync(0xffffffffu, mn[ax], o));
      mx[ax] = max(mx[ax], __shfl_xor_sync(0xffffffffu, mx[ax], o));
    }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int ax = 0; ax < 3; ax++)
    {
      red[ax][w] = mn[ax];
      red[3 + ax][w] = mx[ax];
    }
  __syncthreads();
  if (threadIdx.x < 6)
  {
    const int ax = threadIdx.x;
    int32_t r = ax < 3 ? INT32_MAX : INT32_MIN;
    for (int q = 0; q < kLeafThreads / 32; q++)
      r = ax < 3 ? min(r, red[ax][q]) : max(r, red[ax][q]);
    box[(uint64_t)ax * L + l] = r;
  }
}

/* Records overwritten by a later duplicate point at the survivor's slot. */
__global__ void dupMapKernel(KeyArgs a, const uint64_t *__restrict__ keys, const uint32_t *__restrict__ idx,
                             const uint32_t *__restrict__ surv, uint32_t *__restrict__ storeOf)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += (uint64_t)gridDim.x * blockDim.x)
    if (!surv[i])
    {
      uint64_t k = keys[i];
      uint64_t last = i;
      for (uint64_t j = i + 1; j < a.n && keys[j] == k; j++)
        if (sameDoubles(a, idx[i], idx[j]))
          last = j;
      storeOf[idx[i]] = storeOf[idx[last]];
    }
}

__global__ void pointLeafKernel(uint64_t n, const uint32_t *__restrict__ storeOf, const uint32_t *__restrict__ leafId,
                                uint32_t *__restrict__ pointLeaf)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    pointLeaf[i] = leafId[storeOf[i]];
}

/* ---- node hierarchy ---- */
__global__ void nodeStartKernel(uint64_t L, int D, const uint8_t *__restrict__ leafLev,
                                const uint64_t *__restrict__ leafKey, uint32_t *__restrict__ flag)
{
  uint64_t total = L * (uint64_t)D;
  for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (uint64_t)gridDim.x * blockDim.x)
  {
    int d = (int)(t / L);
    uint64_t l = t % L;
    uint32_t f = 0;
    if (leafLev[l] > d)
      f = (l == 0) || (leafLev[l - 1] <= d) || (prefixAt(leafKey[l - 1], d) != prefixAt(leafKey[l], d));
    flag[t] = f;
  }
}

__device__ __forceinline__ int32_t nodeIdAt(const uint32_t *ex, const uint32_t *flag, uint64_t L, int d, uint64_t l)
{
  uint64_t t = (uint64_t)d * L + l;
  return (int32_t)(ex[t] + flag[t]) - 1;
}

/* child encoding: >=0 internal node, -1 empty, <=-2 leaf (-2 - leaf). */
__global__ void nodeLinkKernel(uint64_t L, int D, const uint8_t *__restrict__ leafLev,
                               const uint64_t *__restrict__ leafKey, const uint32_t *__restrict__ flag,
                               const uint32_t *__restrict__ ex, int32_t *__restrict__ child,
                               const int32_t *__restrict__ leafBox, int32_t *__restrict__ nodeBox, uint64_t N)
{
  for (uint64_t l = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; l < L; l += (uint64_t)gridDim.x * blockDim.x)
  {
    int lv = leafLev[l];
    uint64_t key = leafKey[l];
    int32_t b[6];
#pragma unroll
    for (int k = 0; k < 6; k++)
      b[k] = leafBox[(uint64_t)k * L + l];
    for (int d = 0; d < lv && d < D; d++)
    {
      int32_t nid = nodeIdAt(ex, flag, L, d, l);
      int oct = (int)((key >> (60 - 3 * d)) & 7);
      if (lv == d + 1)
        child[(uint64_t)nid * 8 + oct] = -2 - (int32_t)l;
      else if (flag[(uint64_t)(d + 1) * L + l])
        child[(uint64_t)nid * 8 + oct] = nodeIdAt(ex, flag, L, d + 1, l);
      for (int k = 0; k < 3; k++)
      {
        atomicMin(&nodeBox[(uint64_t)k * N + nid], b[k]);
        atomicMax(&nodeBox[(uint64_t)(3 + k) * N + nid], b[3 + k]);
      }
    }
  }
}

__global__ void fillI32(int32_t *p, uint64_t n, int32_t v)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = v;
}

__global__ void maxLevelKernel(uint64_t L, const uint8_t *__restrict__ leafLev, int *__restrict__ out)
{
  int m = 0;
  for (uint64_t l = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; l < L; l += (uint64_t)gridDim.x * blockDim.x)
    m = max(m, (int)leafLev[l]);
  for (int o = 16; o; o >>= 1)
    m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0)
    atomicMax(out, m);
}

}  // namespace

static unsigned gridFor(wb_ctx *c, uint64_t n, int threads = 256)
{
  uint64_t b = (n + threads - 1) / threads;
  uint64_t cap = (uint64_t)c->sm_count * 16;
  if (b > cap)
    b = cap;
  if (b < 1)
    b = 1;
  return (unsigned)b;
}

/* Sets up the fixed-point cell coordinate of axis k (see KeyArgs).  t is
 * the coordinate in cell units, (decode(X) - lo) / cell, linear in X up to
 * the rounding of decode; the error allowed for (eps) covers the rounding of
 * R and C to 2^-shift, the decode's two roundings and the double arithmetic
 * here, with a factor of 16 to spare. */
static void keyFixedPoint(const WbGeom &g, double mn, double mx, int k, KeyArgs &a)
{
  a.fixed[k] = 0;
  a.shift[k] = 0;
  a.x0[k] = a.dmax[k] = a.rfix[k] = a.cfix[k] = a.eps[k] = 0;
  const double u = g.scale[k] * g.unit;
  if (!(u > 0) || !(g.unit > 0) || !(g.cell > 0))
    return;
  const double R = u / g.cell;   // the cell is a power of two: exact
  double xlo = (fmin(mn, mx) / g.unit - g.off[k]) / g.scale[k], xhi = (fmax(mn, mx) / g.unit - g.off[k]) / g.scale[k];
  if (!(fabs(xlo) < 2e9) || !(fabs(xhi) < 2e9))
    return;
  const long long X0 = llround((xlo + xhi) / 2);
  const long long dmax = (long long)ceil(fmax(fabs(xlo - X0), fabs(xhi - X0))) + 4;
  const double x0d = (g.off[k] + g.scale[k] * (double)X0) * g.unit;
  const double C = (x0d - g.root_lo[k]) / g.cell;
  const double B = fabs(C) + (double)dmax * R + 4;
  int shift = 62 - (int)ceil(log2(B));
  if (shift > 40)
    shift = 40;
  if (shift < 24)
    return;
  const double one = ldexp(1.0, shift);
  // decode error: two roundings of |x| (<= |x0d| + dmax*u) and the subtraction of lo
  const double mag = fabs(x0d) + (double)dmax * u + fabs(g.root_lo[k]);
  const double errCells = (double)dmax / one + 1.0 / one + 8 * ldexp(mag, -52) / g.cell + ldexp(B, -50);
  a.fixed[k] = 1;
  a.shift[k] = shift;
  a.x0[k] = X0;
  a.dmax[k] = dmax;
  a.rfix[k] = llround(R * one);
  a.cfix[k] = llround(C * one);
  a.eps[k] = (long long)ceil(16 * errCells * one) + 16;
}

/* The point -> leaf map of every record (leaf of its store slot), formed when
 * a caller asks for it: the pipeline itself reads store slots only. */
int wb_point_leaf_map(wb_ctx *c)
{
  const uint64_t n = c->n;
  int rc;
  if (!n)
    return 0;
  if ((rc = wb_ensure(c, c->pointLeaf, n * 4 + 64)))
    return rc;
  { pointLeafKernel<<<gridFor(c, n), 256, 0, c->stream>>>(n, (const uint32_t *)c->storeOf.p,
                                                          (const uint32_t *)c->leafId.p, (uint32_t *)c->pointLeaf.p); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  return 0;
}

int wb_build_impl(wb_ctx *c, const wb_cloud *cl)
{
  if (!cl || !cl->records || cl->stride < 12)
    return wb_fail(c, WB_EINVAL, "wb_octree_build: records must be non-null with stride >= 12");
  if (cl->n > 0xfffffff0ull)
    return wb_fail(c, WB_EINVAL, "wb_octree_build: at most 2^32-16 points per cloud");
  uint64_t n = cl->n;
  // with paging, a cloud whose working set (about 340 B per point plus the
  // records) is above the HBM budget keeps its scratch buffers in host memory
  c->spill_cold = c->host_budget && c->budget &&
                  n * (340ull + (cl->device_resident ? 0 : cl->stride)) > c->budget;
  WbGeom &g = c->g;
  for (int a = 0; a < 3; a++)
  {
    g.off[a] = cl->offset[a];
    g.scale[a] = cl->scale[a];
  }
  g.unit = cl->unit;
  double mn[3], mx[3];
  for (int a = 0; a < 3; a++)
  {
    mn[a] = cl->minc[a] * cl->unit;
    mx[a] = cl->maxc[a] * cl->unit;
  }
  wb_size_fit(mn, mx, g.root_c, &g.root_side);
  if (!(g.root_side > 0))
    return wb_fail(c, WB_EINVAL, "wb_octree_build: header min/max enclose no volume");
  for (int a = 0; a < 3; a++)
    g.root_lo[a] = g.root_c[a] - g.root_side / 2;
  g.cell = ldexp(g.root_side, -WB_LEVELS);
  wb_tile_cube(mn, mx, g.tile_c, &g.tile_side);
  c->n = n;
  c->stage = 0;

  KeyArgs a;
  a.n = n;
  a.stride = cl->stride;
  for (int k = 0; k < 3; k++)
  {
    a.off[k] = g.off[k];
    a.scale[k] = g.scale[k];
    a.lo[k] = g.root_lo[k];
  }
  a.unit = g.unit;
  a.cell = g.cell;
  for (int k = 0; k < 3; k++)
    keyFixedPoint(g, mn[k], mx[k], k, a);

  int rc;
  if (cl->device_resident && n && !wb_device_accessible(cl->records))
    return wb_fail(c, WB_EINVAL, "wb_octree_build: device_resident records must be device memory");
  if (cl->device_resident)
    a.rec = (const uint8_t *)cl->records;
  else
  {
    if ((rc = wb_ensure(c, c->rec, n * (uint64_t)cl->stride)))
      return rc;
    if ((rc = wb_copy_in(c, c->rec.p, cl->records, n * (uint64_t)cl->stride)))
      return rc;
    a.rec = (const uint8_t *)c->rec.p;
  }
  wb_mark(c, "upload");
  if (n == 0)
  {
    c->nd = c->n_leaves = c->n_nodes = 0;
    c->stage = 1;
    return 0;
  }
  if ((rc = wb_ensure(c, c->key0, n * 8)) || (rc = wb_ensure(c, c->key1, n * 8)) ||
      (rc = wb_ensure(c, c->idx0, n * 4)) || (rc = wb_ensure(c, c->idx1, n * 4)) ||
      (rc = wb_ensure(c, c->tmp32, n * 4)) || (rc = wb_ensure(c, c->storeOf, n * 4)) ||
      (rc = wb_ensure(c, c->survivorOf, n * 4)) ||
      (rc = wb_ensure(c, c->small, 4096)))
    return rc;
  uint64_t *keys = (uint64_t *)c->key0.p;
  uint32_t *idx = (uint32_t *)c->idx0.p;
  { keyKernel<<<gridFor(c, n), 256, 0, c->stream>>>(a, keys, idx); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  wb_mark(c, "decode_key");
  uint64_t *kAlt = (uint64_t *)c->key1.p;
  uint32_t *iAlt = (uint32_t *)c->idx1.p;
  if ((rc = wb_radix_sort_pairs(c, keys, idx, kAlt, iAlt, n, 0, 63)))
    return rc;
  kAlt = (keys == (uint64_t *)c->key0.p) ? (uint64_t *)c->key1.p : (uint64_t *)c->key0.p;
  iAlt = (idx == (uint32_t *)c->idx0.p) ? (uint32_t *)c->idx1.p : (uint32_t *)c->idx0.p;
  wb_mark(c, "sort");

  uint32_t *surv = (uint32_t *)c->tmp32.p;
  uint32_t *rank = (uint32_t *)c->survivorOf.p;   // scratch: survivor rank
  int *dErr = (int *)c->small.p;
  uint32_t *dTot = (uint32_t *)((char *)c->small.p + 64);
  int *dMax = (int *)((char *)c->small.p + 128);
  WB_CUDA(c, cudaMemsetAsync(c->small.p, 0, 256, c->stream));
  { survivorKernel<<<gridFor(c, n), 256, 0, c->stream>>>(a, keys, idx, surv); ++c->launches; }
  if ((rc = wb_exclusive_scan_u32(c, surv, rank, n, dTot)))
    return rc;
  uint32_t ndh = 0;
  WB_CUDA(c, cudaMemcpyAsync(&ndh, dTot, 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  uint64_t nd = ndh;
  c->nd = nd;
  uint64_t *dkey = kAlt;
  uint32_t *didx = iAlt;
  { compactKernel<<<gridFor(c, n), 256, 0, c->stream>>>(n, keys, idx, surv, rank, dkey, didx); ++c->launches; }
  wb_mark(c, "dedup");

  uint64_t nw = nd >= (uint64_t)kWindow ? nd - kWindow + 1 : 0;
  if ((rc = wb_ensure(c, c->cpl, nw + 64)) || (rc = wb_ensure(c, c->pre, nw + 64)) ||
      (rc = wb_ensure(c, c->suf, nw + 64)) || (rc = wb_ensure(c, c->lev, nd + 64)) ||
      (rc = wb_ensure(c, c->leafId, nd * 4 + 64)) || (rc = wb_ensure(c, c->tmp32b, nd * 4 * 2 + 64)))
    return rc;
  uint8_t *cpl = (uint8_t *)c->cpl.p, *pre = (uint8_t *)c->pre.p, *suf = (uint8_t *)c->suf.p;
  uint8_t *lev = (uint8_t *)c->lev.p;
  if (nw)
  {
    { cplKernel<<<gridFor(c, nw), 256, 0, c->stream>>>(dkey, nw, cpl); ++c->launches; }
    uint64_t segs = (nw + kWindow - 1) / kWindow;
    { segMaxKernel<<<(unsigned)((segs * 32 + 255) / 256), 256, 0, c->stream>>>(cpl, nw, pre, suf); ++c->launches; }
  }
  { levelKernel<<<gridFor(c, nd), 256, 0, c->stream>>>(nd, nw, pre, suf, lev, dErr); ++c->launches; }
  uint32_t *start = (uint32_t *)c->tmp32b.p;
  uint32_t *startEx = start + nd;
  { leafStartKernel<<<gridFor(c, nd), 256, 0, c->stream>>>(nd, dkey, lev, start); ++c->launches; }
  if ((rc = wb_exclusive_scan_u32(c, start, startEx, nd, dTot)))
    return rc;
  uint32_t Lh = 0;
  int errh = 0;
  WB_CUDA(c, cudaMemcpyAsync(&Lh, dTot, 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaMemcpyAsync(&errh, dErr, 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (errh)
    return wb_fail(c, WB_EDEPTH, "wb_octree_build: more than 537 distinct points in a cell 21 levels below the root");
  uint64_t L = Lh;
  c->n_leaves = L;
  if ((rc = wb_ensure(c, c->leafFirst, L * 4 + 64)) || (rc = wb_ensure(c, c->leafCount, L * 4 + 64)) ||
      (rc = wb_ensure(c, c->leafLevel, L + 64)) || (rc = wb_ensure(c, c->leafKey, L * 8 + 64)) ||
      (rc = wb_ensure(c, c->leafBox, L * 24 + 64)) || (rc = wb_ensure(c, c->sidx, nd * 4 + 64)) ||
      (rc = wb_ensure(c, c->sx, nd * 4 + 64)) || (rc = wb_ensure(c, c->sy, nd * 4 + 64)) ||
      (rc = wb_ensure(c, c->sz, nd * 4 + 64)) || (rc = wb_ensure(c, c->xyzd, nd * 24 + 64)))
    return rc;
  uint32_t *leafId = (uint32_t *)c->leafId.p, *first = (uint32_t *)c->leafFirst.p, *count = (uint32_t *)c->leafCount.p;
  uint8_t *leafLev = (uint8_t *)c->leafLevel.p;
  uint64_t *leafKey = (uint64_t *)c->leafKey.p;
  { leafTableKernel<<<gridFor(c, nd), 256, 0, c->stream>>>(nd, dkey, lev, start, startEx, leafId, first, leafLev, leafKey); ++c->launches; }
  { leafCountKernel<<<gridFor(c, L), 256, 0, c->stream>>>(L, nd, first, count); ++c->launches; }
  wb_mark(c, "leaves");
  int32_t *box = (int32_t *)c->leafBox.p;
  uint32_t *storeOf = (uint32_t *)c->storeOf.p;
  { leafSortKernel<<<(unsigned)L, kLeafThreads, 0, c->stream>>>(a, first, count, didx, (uint32_t *)c->sidx.p,
                                                               (int32_t *)c->sx.p, (int32_t *)c->sy.p, (int32_t *)c->sz.p,
                                                               box, storeOf, L,
                                                               (double *)c->xyzd.p, nd); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  wb_mark(c, "leaf_order");
  // records a later identical point overwrote take their survivor's slot
  if (nd != n)
  {
    { dupMapKernel<<<gridFor(c, n), 256, 0, c->stream>>>(a, keys, idx, surv, storeOf); ++c->launches; }
  }
  { maxLevelKernel<<<gridFor(c, L), 256, 0, c->stream>>>(L, leafLev, dMax); ++c->launches; }
  int maxLev = 0;
  WB_CUDA(c, cudaMemcpyAsync(&maxLev, dMax, 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  c->max_depth = (uint32_t)maxLev;
  wb_mark(c, "point_map");

  // node hierarchy over levels 0 .. maxLev-1
  int D = maxLev;
  uint64_t LD = L * (uint64_t)D;
  if ((rc = wb_ensure(c, c->nodeStart, LD * 8 + 64)))
    return rc;
  uint32_t *flag = (uint32_t *)c->nodeStart.p;
  uint32_t *flagEx = flag + LD;
  { nodeStartKernel<<<gridFor(c, LD), 256, 0, c->stream>>>(L, D, leafLev, leafKey, flag); ++c->launches; }
  if ((rc = wb_exclusive_scan_u32(c, flag, flagEx, LD, dTot)))
    return rc;
  uint32_t Nh = 0;
  WB_CUDA(c, cudaMemcpyAsync(&Nh, dTot, 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  uint64_t N = Nh;
  c->n_nodes = N;
  if ((rc = wb_ensure(c, c->nodeChild, N * 32 + 64)) || (rc = wb_ensure(c, c->nodeBox, N * 24 + 64)))
    return rc;
  int32_t *child = (int32_t *)c->nodeChild.p, *nbox = (int32_t *)c->nodeBox.p;
  { fillI32<<<gridFor(c, N * 8), 256, 0, c->stream>>>(child, N * 8, -1); ++c->launches; }
  { fillI32<<<gridFor(c, N * 3), 256, 0, c->stream>>>(nbox, N * 3, INT32_MAX); ++c->launches; }
  { fillI32<<<gridFor(c, N * 3), 256, 0, c->stream>>>(nbox + N * 3, N * 3, INT32_MIN); ++c->launches; }
  { nodeLinkKernel<<<gridFor(c, L), 256, 0, c->stream>>>(L, D, leafLev, leafKey, flag, flagEx, child, box, nbox, N); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  wb_mark(c, "nodes");
  c->grid_bounds[0] = mn[0];
  c->grid_bounds[1] = mn[1];
  c->grid_bounds[2] = mx[0];
  c->grid_bounds[3] = mx[1];
  if ((rc = wb_grid_impl(c, mn[0], mn[1], mx[0], mx[1])))
    return rc;
  wb_mark(c, "grid");
  c->stage = 1;
  return 0;
}

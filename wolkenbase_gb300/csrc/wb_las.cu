/* The steps either side of the path: LAS class bytes and the class split,
 * class totals and the duplicate report.
 *
 *  wb_class_totals       OctStore::countClasses over every block
 *                        (octree.cpp:664-671, 878-881; threads.cpp:425-444)
 *  wb_duplicates         OctBuffer::put's overwrite of an identical point
 *                        (octree.cpp:620-662), counted as alreadyInOctree
 *  wb_las_write_classes  the classification field LasHeader::writePoint
 *                        writes (las.cpp:853-862): formats 0-5 keep the three
 *                        flag bits above the 5-bit class, 6-10 the whole byte
 *  wb_las_split_by_class CloudOutput::writeFiles's grouping of the points by
 *                        class (cloudoutput.cpp:187-231): a stable partition
 *                        of the records on the device; the files are the
 *                        caller's
 *  wb_preview            OctStore::hiLoPointsIn / countPointsIn over the
 *                        pixel columns of a view (octree.cpp:1244-1293)
 *
 * All of it is byte movement: one pass of HBM reads and writes per kernel,
 * records copied with the widest loads their stride allows.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>
#include "wb_internal.h"

namespace
{
/* Byte offset of the class field in a LAS point record (las.cpp:747-773). */
__host__ __device__ __forceinline__ int classOffset(int format)
{
  return format < 6 ? 15 : 16;
}

__device__ __forceinline__ uint8_t classOf(const uint8_t *rec, int format)
{
  uint8_t b = rec[classOffset(format)];
  return format < 6 ? (uint8_t)(b & 31) : b;
}

__global__ void classTotalsKernel(uint64_t nd, const uint32_t *__restrict__ sidx, const uint8_t *__restrict__ cls,
                                  unsigned long long *__restrict__ totals)
{
  __shared__ unsigned int h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    h[i] = 0;
  __syncthreads();
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nd; j += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(&h[cls[sidx[j]]], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i])
      atomicAdd(&totals[i], (unsigned long long)h[i]);
}

__global__ void dupKernel(uint64_t n, const uint32_t *__restrict__ storeOf, const uint32_t *__restrict__ sidx,
                          uint32_t *__restrict__ dupOf)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    dupOf[i] = sidx[storeOf[i]];
}

__global__ void writeClassesKernel(uint8_t *__restrict__ rec, uint64_t n, uint32_t stride, int format,
                                   const uint8_t *__restrict__ cls)
{
  const int off = classOffset(format);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint8_t *b = rec + i * stride + off;
    *b = format < 6 ? (uint8_t)((*b & 0xe0) | (cls[i] & 31)) : cls[i];
  }
}

/* Class of every record as a sort key, its index as the value. */
__global__ void classKeysKernel(const uint8_t *__restrict__ rec, uint64_t n, uint32_t stride, int format,
                                uint64_t *__restrict__ keys, uint32_t *__restrict__ idx,
                                unsigned long long *__restrict__ hist)
{
  __shared__ unsigned int h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    h[i] = 0;
  __syncthreads();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    uint8_t c = classOf(rec + i * stride, format);
    keys[i] = c;
    idx[i] = (uint32_t)i;
    atomicAdd(&h[c], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i])
      atomicAdd(&hist[i], (unsigned long long)h[i]);
}

/* out record k = in record perm[k], one thread per record, copied in words
 * of the widest size the stride and both bases allow. */
template <typename Word>
__global__ void gatherRecordsKernel(const uint8_t *__restrict__ in, uint8_t *__restrict__ out, uint64_t n,
                                    uint32_t stride, const uint32_t *__restrict__ perm)
{
  const uint32_t words = stride / (uint32_t)sizeof(Word);
  for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
  {
    const Word *src = (const Word *)(in + (uint64_t)perm[k] * stride);
    Word *dst = (Word *)(out + k * stride);
    for (uint32_t w = 0; w < words; w++)
      dst[w] = src[w];
  }
}

/* Stable partition of records by class byte, in two passes over tiles of
 * kPartTile records: partCount writes each tile's class counts (class-major,
 * so one scan gives every (class, tile) its first output record), and
 * partScatter re-reads the tile, ranks its records within their class in
 * input order (warps walk their records in order with match_any), and copies
 * them word by word into the class runs of the output: consecutive threads
 * write consecutive words of a run. */
constexpr int kPartThreads = 256, kPartPer = 8, kPartTile = kPartThreads * kPartPer;

__global__ void __launch_bounds__(kPartThreads) partCount(const uint8_t *__restrict__ rec, uint64_t n,
                                                          uint32_t stride, int format, uint32_t numTiles,
                                                          uint32_t *__restrict__ counts,
                                                          unsigned long long *__restrict__ hist)
{
  __shared__ unsigned int h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    h[i] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * kPartTile;
  for (int k = 0; k < kPartPer; k++)
  {
    const uint64_t i = base + (uint64_t)k * kPartThreads + threadIdx.x;
    if (i < n)
      atomicAdd(&h[classOf(rec + i * stride, format)], 1u);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < 256; c += blockDim.x)
  {
    counts[(uint64_t)c * numTiles + blockIdx.x] = h[c];
    if (h[c])
      atomicAdd(&hist[c], (unsigned long long)h[c]);
  }
}

__global__ void __launch_bounds__(kPartThreads) partScatter(const uint8_t *__restrict__ rec, uint64_t n,
                                                            uint32_t stride, int format, uint32_t numTiles,
                                                            const uint32_t *__restrict__ offs,
                                                            uint8_t *__restrict__ out)
{
  constexpr int W = kPartThreads / 32;
  __shared__ uint32_t wcount[W][256];
  __shared__ uint32_t localStart[256], globalStart[256];
  __shared__ uint32_t order[kPartTile];   // tile record of each local (class-sorted) position
  __shared__ uint8_t clsOf[kPartTile];    // class of each local position
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < W * 256; i += kPartThreads)
    (&wcount[0][0])[i] = 0;
  __syncthreads();
  const uint64_t tbase = (uint64_t)blockIdx.x * kPartTile;
  const uint32_t tileN = (uint32_t)(n - tbase < (uint64_t)kPartTile ? n - tbase : (uint64_t)kPartTile);
  uint32_t rank[kPartPer];
  uint8_t cl[kPartPer];
  const unsigned lt = (1u << lane) - 1;
  // warp w takes records [w*256, (w+1)*256) of the tile, 32 at a time, in order
#pragma unroll
  for (int q = 0; q < kPartPer; q++)
  {
    const uint32_t r = (uint32_t)warp * (kPartPer * 32) + q * 32 + lane;
    const bool ok = r < tileN;
    const uint32_t d = ok ? classOf(rec + (tbase + r) * stride, format) : 256u;
    cl[q] = (uint8_t)d;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t pre = d < 256 ? wcount[warp][d] : 0;
    rank[q] = pre + __popc(peers & lt);
    __syncwarp();
    if (d < 256 && (peers & lt) == 0)
      wcount[warp][d] = pre + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kPartThreads)
  {
    uint32_t run = 0;
    for (int w = 0; w < W; w++)
    {
      const uint32_t c = wcount[w][d];
      wcount[w][d] = run;
      run += c;
    }
    localStart[d] = run;
    globalStart[d] = offs[(uint64_t)d * numTiles + blockIdx.x];
  }
  __syncthreads();
  if (warp == 0)
  {
    uint32_t c[8], sum = 0;
#pragma unroll
    for (int q = 0; q < 8; q++)
    {
      c[q] = localStart[lane * 8 + q];
      sum += c[q];
    }
    uint32_t inc = sum;
    for (int o = 1; o < 32; o <<= 1)
    {
      const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o)
        inc += v;
    }
    uint32_t run = inc - sum;
#pragma unroll
    for (int q = 0; q < 8; q++)
    {
      localStart[lane * 8 + q] = run;
      run += c[q];
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < kPartPer; q++)
  {
    const uint32_t r = (uint32_t)warp * (kPartPer * 32) + q * 32 + lane;
    if (r < tileN)
    {
      const uint32_t lp = localStart[cl[q]] + wcount[warp][cl[q]] + rank[q];
      order[lp] = r;
      clsOf[lp] = cl[q];
    }
  }
  __syncthreads();
  // copy: word w of the tile's class-ordered records goes to its class run
  const uint32_t words = stride / 4;
  const uint64_t total = (uint64_t)tileN * words;
  auto copyWord = [&](uint32_t lp, uint32_t k) {
    const uint32_t d = clsOf[lp];
    const uint64_t dst = (uint64_t)globalStart[d] + (lp - localStart[d]);
    ((uint32_t *)out)[dst * words + k] = ((const uint32_t *)rec)[(tbase + order[lp]) * words + k];
  };
  if (words > 1 && total * words < (1ull << 32))
  {
    // w / words as the high half of w * ceil(2^32 / words): exact while
    // w * words < 2^32 (the rounding of the reciprocal stays below 1 / words)
    const uint32_t magic = (uint32_t)(((1ull << 32) + words - 1) / words);
    for (uint32_t w = threadIdx.x; w < (uint32_t)total; w += kPartThreads)
    {
      const uint32_t lp = __umulhi(w, magic);
      copyWord(lp, w - lp * words);
    }
  }
  else
    for (uint64_t w = threadIdx.x; w < total; w += kPartThreads)
      copyWord((uint32_t)(w / words), (uint32_t)(w % words));
}

unsigned gridOf(const wb_ctx *c, uint64_t n)
{
  return (unsigned)std::min<uint64_t>((n + 255) / 256 + 1, (uint64_t)c->sm_count * 16);
}
}  // namespace

extern "C" {

int wb_class_totals(wb_ctx *c, uint64_t *totals)
{
  if (!c || !totals)
    return WB_EINVAL;
  if (c->stage < 3 || !c->clsFinal)
    return wb_fail(c, WB_ESTATE, "wb_class_totals: classify first");
  WbDeviceGuard deviceGuard(c->device);
  WbScratch out(c);
  int rc = wb_ensure(c, out.b, 256 * 8);
  if (rc)
    return rc;
  WB_CUDA(c, cudaMemsetAsync(out.b.p, 0, 256 * 8, c->stream));
  if (c->nd)
    { classTotalsKernel<<<gridOf(c, c->nd), 256, 0, c->stream>>>(c->nd, (const uint32_t *)c->sidx.p, c->clsFinal,
                                                                  (unsigned long long *)out.b.p); ++c->launches; }
  cudaError_t e = cudaMemcpyAsync(totals, out.b.p, 256 * 8, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess)
    return wb_fail(c, WB_ECUDA, std::string("wb_class_totals: ") + cudaGetErrorString(e));
  return 0;
}

int wb_duplicates(wb_ctx *c, uint64_t *n_dup, uint32_t *dup_of)
{
  if (!c || !n_dup)
    return WB_EINVAL;
  if (c->stage < 1)
    return wb_fail(c, WB_ESTATE, "wb_duplicates: build the octree first");
  *n_dup = c->n - c->nd;
  if (!dup_of || !c->n)
    return 0;
  WbDeviceGuard deviceGuard(c->device);
  WbScratch out(c);
  int rc = wb_ensure(c, out.b, c->n * 4);
  if (rc)
    return rc;
  { dupKernel<<<gridOf(c, c->n), 256, 0, c->stream>>>(c->n, (const uint32_t *)c->storeOf.p,
                                                       (const uint32_t *)c->sidx.p, (uint32_t *)out.b.p); ++c->launches; }
  cudaError_t e = cudaMemcpyAsync(dup_of, out.b.p, c->n * 4, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess)
    return wb_fail(c, WB_ECUDA, std::string("wb_duplicates: ") + cudaGetErrorString(e));
  return 0;
}

int wb_las_write_classes(wb_ctx *c, void *records, uint64_t n, uint32_t stride, int point_format, int on_device,
                         const uint8_t *cls)
{
  if (!c || (n && !records))
    return WB_EINVAL;
  if (point_format < 0 || point_format > 10 || stride < (uint32_t)classOffset(point_format) + 1)
    return wb_fail(c, WB_EINVAL, "wb_las_write_classes: point format 0-10 and a stride that holds its class field");
  if (!cls && (c->stage < 3 || !c->clsFinal || n != c->n))
    return wb_fail(c, WB_ESTATE, "wb_las_write_classes: no class bytes of a classified cloud of n records");
  if (!n)
    return 0;
  if (on_device && (!wb_device_accessible(records) || (cls && !wb_device_accessible(cls))))
    return wb_fail(c, WB_EINVAL, "wb_las_write_classes: on_device needs device pointers");
  WbDeviceGuard deviceGuard(c->device);
  int rc;
  WbScratch rbuf(c), cbuf(c);
  uint8_t *drec = (uint8_t *)records;
  const uint8_t *dcls = cls ? cls : c->clsFinal;
  if (!on_device)
  {
    if ((rc = wb_ensure(c, rbuf.b, n * stride)))
      return rc;
    drec = (uint8_t *)rbuf.b.p;
    WB_CUDA(c, cudaMemcpyAsync(drec, records, n * stride, cudaMemcpyDefault, c->stream));
    if (cls)
    {
      if ((rc = wb_ensure(c, cbuf.b, n)))
        return rc;
      WB_CUDA(c, cudaMemcpyAsync(cbuf.b.p, cls, n, cudaMemcpyDefault, c->stream));
      dcls = (const uint8_t *)cbuf.b.p;
    }
  }
  { writeClassesKernel<<<gridOf(c, n), 256, 0, c->stream>>>(drec, n, stride, point_format, dcls); ++c->launches; }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && !on_device)
    e = cudaMemcpyAsync(records, drec, n * stride, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess)
    return wb_fail(c, WB_ECUDA, std::string("wb_las_write_classes: ") + cudaGetErrorString(e));
  return 0;
}

int wb_las_split_by_class(wb_ctx *c, const void *records, uint64_t n, uint32_t stride, int point_format,
                          int on_device, void *out, uint64_t *offsets)
{
  if (!c || !offsets || (n && (!records || !out)))
    return WB_EINVAL;
  if (point_format < 0 || point_format > 10 || stride < (uint32_t)classOffset(point_format) + 1)
    return wb_fail(c, WB_EINVAL, "wb_las_split_by_class: point format 0-10 and a stride that holds its class field");
  if (n >= 0xffffffffull)
    return wb_fail(c, WB_EINVAL, "wb_las_split_by_class: at most 2^32-1 records");
  memset(offsets, 0, 257 * sizeof(uint64_t));
  if (!n)
    return 0;
  if (on_device && (!wb_device_accessible(records) || !wb_device_accessible(out)))
    return wb_fail(c, WB_EINVAL, "wb_las_split_by_class: on_device needs device pointers");
  WbDeviceGuard deviceGuard(c->device);
  int rc;
  WbScratch rin(c), rout(c), hist(c);
  const uint8_t *din = (const uint8_t *)records;
  uint8_t *dout = (uint8_t *)out;
  if (!on_device)
  {
    if ((rc = wb_ensure(c, rin.b, n * stride)) || (rc = wb_ensure(c, rout.b, n * stride)))
      return rc;
    WB_CUDA(c, cudaMemcpyAsync(rin.b.p, records, n * stride, cudaMemcpyDefault, c->stream));
    din = (const uint8_t *)rin.b.p;
    dout = (uint8_t *)rout.b.p;
  }
  if ((rc = wb_ensure(c, hist.b, 256 * 8)))
    return rc;
  WB_CUDA(c, cudaMemsetAsync(hist.b.p, 0, 256 * 8, c->stream));
  if (stride % 4 == 0 && ((uintptr_t)din % 4 == 0) && ((uintptr_t)dout % 4 == 0))
  {
    // the stable partition: records read twice in order, written once
    const uint64_t numTiles = (n + kPartTile - 1) / kPartTile;
    WbScratch cnt(c), off(c);
    if ((rc = wb_ensure(c, cnt.b, numTiles * 256 * 4 + 64)) || (rc = wb_ensure(c, off.b, numTiles * 256 * 4 + 64)))
      return rc;
    { partCount<<<(unsigned)numTiles, kPartThreads, 0, c->stream>>>(din, n, stride, point_format, (uint32_t)numTiles,
                                                                   (uint32_t *)cnt.b.p,
                                                                   (unsigned long long *)hist.b.p); ++c->launches; }
    if ((rc = wb_exclusive_scan_u32(c, (const uint32_t *)cnt.b.p, (uint32_t *)off.b.p, numTiles * 256, nullptr)))
      return rc;
    { partScatter<<<(unsigned)numTiles, kPartThreads, 0, c->stream>>>(din, n, stride, point_format, (uint32_t)numTiles,
                                                                     (const uint32_t *)off.b.p, dout); ++c->launches; }
    uint64_t h[256];
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(h, hist.b.p, sizeof h, cudaMemcpyDefault, c->stream);
    if (e == cudaSuccess && !on_device)
      e = cudaMemcpyAsync(out, dout, n * stride, cudaMemcpyDefault, c->stream);
    if (e == cudaSuccess)
      e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess)
      return wb_fail(c, WB_ECUDA, std::string("wb_las_split_by_class: ") + cudaGetErrorString(e));
    for (int k = 0; k < 256; k++)
      offsets[k + 1] = offsets[k] + h[k];
    return 0;
  }
  // strides or bases that are not word multiples: class keys, one radix pass, a record gather
  if ((rc = wb_ensure(c, c->key0, n * 8)) || (rc = wb_ensure(c, c->key1, n * 8)) ||
      (rc = wb_ensure(c, c->idx0, n * 4)) || (rc = wb_ensure(c, c->idx1, n * 4)))
    return rc;
  uint64_t *keys = (uint64_t *)c->key0.p;
  uint32_t *idx = (uint32_t *)c->idx0.p;
  { classKeysKernel<<<gridOf(c, n), 256, 0, c->stream>>>(din, n, stride, point_format, keys, idx,
                                                         (unsigned long long *)hist.b.p); ++c->launches; }
  // one stable pass of the 8-bit digit: records keep their order within a class
  if ((rc = wb_radix_sort_pairs(c, keys, idx, (uint64_t *)c->key1.p, (uint32_t *)c->idx1.p, n, 0, 8)))
    return rc;
  if (stride % 16 == 0 && ((uintptr_t)din % 16 == 0) && ((uintptr_t)dout % 16 == 0))
    { gatherRecordsKernel<uint4><<<gridOf(c, n), 256, 0, c->stream>>>(din, dout, n, stride, idx); ++c->launches; }
  else if (stride % 8 == 0 && ((uintptr_t)din % 8 == 0) && ((uintptr_t)dout % 8 == 0))
    { gatherRecordsKernel<uint2><<<gridOf(c, n), 256, 0, c->stream>>>(din, dout, n, stride, idx); ++c->launches; }
  else if (stride % 4 == 0 && ((uintptr_t)din % 4 == 0) && ((uintptr_t)dout % 4 == 0))
    { gatherRecordsKernel<uint32_t><<<gridOf(c, n), 256, 0, c->stream>>>(din, dout, n, stride, idx); ++c->launches; }
  else
    { gatherRecordsKernel<uint8_t><<<gridOf(c, n), 256, 0, c->stream>>>(din, dout, n, stride, idx); ++c->launches; }
  uint64_t h[256];
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h, hist.b.p, sizeof h, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess && !on_device)
    e = cudaMemcpyAsync(out, dout, n * stride, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess)
    return wb_fail(c, WB_ECUDA, std::string("wb_las_split_by_class: ") + cudaGetErrorString(e));
  for (int k = 0; k < 256; k++)
    offsets[k + 1] = offsets[k] + h[k];
  return 0;
}

}  // extern "C"

/* ---- Preview queries: OctStore::hiLoPointsIn and countPointsIn (octree.cpp:1244-1293) over
 * the pixels of a view, each pixel a Column (shape.cpp:245-254: an infinitely tall square
 * prism, |cx - x| <= side/2 and |cy - y| <= side/2, both in double) ----
 *
 * WolkenCanvas::pixelColorRead (wolkencanvas.cpp:91-106) asks one pixel at a time; here every
 * stored point visits the pixels whose column can hold it (its nearest pixel centre and, on a
 * boundary, the neighbours), tests them with the reference's comparison, and updates the
 * pixel's count and lowest and highest record Z (decoding is monotone in Z, so the extreme
 * integers decode to the extreme elevations). */
namespace
{
struct ViewArgs
{
  double x0, y0, side;   /* centre of pixel (0, 0) and the pixel size */
  int w, h;
  double off[3], scale[3], unit;
};

__global__ void previewKernel(ViewArgs v, uint64_t nd, const int32_t *__restrict__ sx, const int32_t *__restrict__ sy,
                              const int32_t *__restrict__ sz, unsigned long long *__restrict__ count,
                              int *__restrict__ zlo, int *__restrict__ zhi)
{
  const double half = v.side / 2;
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nd; j += (uint64_t)gridDim.x * blockDim.x)
  {
    const double px = (v.off[0] + v.scale[0] * (double)sx[j]) * v.unit;
    const double py = (v.off[1] + v.scale[1] * (double)sy[j]) * v.unit;
    const double fi = rint((px - v.x0) / v.side), fj = rint((py - v.y0) / v.side);
    if (!(fi > -2 && fi < v.w + 1 && fj > -2 && fj < v.h + 1))
      continue;
    const int i0 = (int)fi, j0 = (int)fj;
    for (int dj = -1; dj <= 1; dj++)
      for (int di = -1; di <= 1; di++)
      {
        const int i = i0 + di, jj = j0 + dj;
        if (i < 0 || i >= v.w || jj < 0 || jj >= v.h)
          continue;
        const double cx = v.x0 + i * v.side, cy = v.y0 + jj * v.side;
        if (fabs(cx - px) <= half && fabs(cy - py) <= half)
        {
          const uint64_t pix = (uint64_t)jj * v.w + i;
          atomicAdd(&count[pix], 1ull);
          atomicMin(&zlo[pix], sz[j]);
          atomicMax(&zhi[pix], sz[j]);
        }
      }
  }
}

__global__ void previewInit(uint64_t npix, unsigned long long *count, int *zlo, int *zhi)
{
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (uint64_t)gridDim.x * blockDim.x)
  {
    count[p] = 0;
    zlo[p] = INT32_MAX;
    zhi[p] = INT32_MIN;
  }
}
}  // namespace

extern "C" int wb_preview(wb_ctx *c, double x0, double y0, double side, int w, int h, uint64_t *count, double *lo,
                          double *hi)
{
  if (!c || w <= 0 || h <= 0 || !(side > 0))
    return WB_EINVAL;
  if (c->stage < 1)
    return wb_fail(c, WB_ESTATE, "wb_preview: build the octree first");
  if (!(c->g.scale[2] * c->g.unit > 0))
    return wb_fail(c, WB_EINVAL, "wb_preview: needs a positive z scale (elevation increasing in Z)");
  WbDeviceGuard deviceGuard(c->device);
  const uint64_t npix = (uint64_t)w * h;
  WbScratch cnt(c), zl(c), zh(c);
  int rc;
  if ((rc = wb_ensure(c, cnt.b, npix * 8)) || (rc = wb_ensure(c, zl.b, npix * 4)) || (rc = wb_ensure(c, zh.b, npix * 4)))
    return rc;
  ViewArgs v;
  v.x0 = x0;
  v.y0 = y0;
  v.side = side;
  v.w = w;
  v.h = h;
  for (int k = 0; k < 3; k++)
  {
    v.off[k] = c->g.off[k];
    v.scale[k] = c->g.scale[k];
  }
  v.unit = c->g.unit;
  { previewInit<<<gridOf(c, npix), 256, 0, c->stream>>>(npix, (unsigned long long *)cnt.b.p, (int *)zl.b.p,
                                                        (int *)zh.b.p); ++c->launches; }
  if (c->nd)
    { previewKernel<<<gridOf(c, c->nd), 256, 0, c->stream>>>(v, c->nd, (const int32_t *)c->sx.p, (const int32_t *)c->sy.p,
                                                              (const int32_t *)c->sz.p, (unsigned long long *)cnt.b.p,
                                                              (int *)zl.b.p, (int *)zh.b.p); ++c->launches; }
  std::vector<int> zlo(npix), zhi(npix);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && count)
    e = cudaMemcpyAsync(count, cnt.b.p, npix * 8, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(zlo.data(), zl.b.p, npix * 4, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(zhi.data(), zh.b.p, npix * 4, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess)
    return wb_fail(c, WB_ECUDA, std::string("wb_preview: ") + cudaGetErrorString(e));
  const WbGeom &g = c->g;
  for (uint64_t p = 0; p < npix; p++)
  {
    // hiLoPointsIn returns (INFINITY, -INFINITY) for an empty shape
    if (lo)
      lo[p] = zlo[p] == INT32_MAX ? INFINITY : (g.off[2] + g.scale[2] * (double)zlo[p]) * g.unit;
    if (hi)
      hi[p] = zhi[p] == INT32_MIN ? -INFINITY : (g.off[2] + g.scale[2] * (double)zhi[p]) * g.unit;
  }
  return 0;
}

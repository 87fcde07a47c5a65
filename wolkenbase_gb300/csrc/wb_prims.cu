/* Device-wide primitives written for this library: exclusive scan of u32 and
 * a stable LSD radix sort of (u64 key, u32 value) pairs.
 *
 * Radix sort: 8-bit digits.  Per pass, one kernel counts digits per tile of
 * 4096 keys, the digit-major count table is scanned, and a second kernel
 * ranks each key inside its tile with warp __match_any_sync groups (stable:
 * a warp walks its 512 keys in order, 32 at a time) and scatters.  Passes
 * whose digit is constant over all keys are skipped.
 */
#include <cuda_runtime.h>
#include <cstdint>
#include "wb_internal.h"

namespace
{
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warpInclusive(uint32_t v)
{
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1)
  {
    uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o)
      v += t;
  }
  return v;
}

/* Block-wide exclusive scan of kScanTile values; writes block total. */
__global__ void scanTiles(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, uint64_t n,
                          uint32_t *__restrict__ blockSums)
{
  __shared__ uint32_t warpSums[32];
  uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
  {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = warpInclusive(s);
  if (lane == 31)
    warpSums[warp] = inc;
  __syncthreads();
  if (warp == 0)
  {
    uint32_t w = warpSums[lane];
    uint32_t wi = warpInclusive(w);
    warpSums[lane] = wi - w;
    if (lane == 31 && blockSums)
      blockSums[blockIdx.x] = wi;
  }
  __syncthreads();
  uint32_t run = inc - s + warpSums[warp];
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
  {
    if (base + k < n)
      out[base + k] = run;
    run += v[k];
  }
}

__global__ void addOffsets(uint32_t *__restrict__ out, uint64_t n, const uint32_t *__restrict__ offs)
{
  uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
  uint32_t add = offs[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; k++)
    if (base + k < n)
      out[base + k] += add;
}

__global__ void totalOf(const uint32_t *in, const uint32_t *ex, uint64_t n, uint32_t *total)
{
  *total = n ? ex[n - 1] + in[n - 1] : 0;
}

/* ---------------- radix sort ---------------- */
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortPerLane = 8;
constexpr int kSortTile = kSortThreads * kSortPerLane;   // 2048

__global__ void __launch_bounds__(kSortThreads) digitCounts(const uint64_t *__restrict__ keys, uint64_t n,
                                                           int shift, uint32_t *__restrict__ counts,
                                                           int numTiles)
{
  __shared__ uint32_t h[256];
  for (int i = threadIdx.x; i < 256; i += kSortThreads)
    h[i] = 0;
  __syncthreads();
  uint64_t base = (uint64_t)blockIdx.x * kSortTile;
  for (int k = 0; k < kSortPerLane; k++)
  {
    uint64_t i = base + (uint64_t)k * kSortThreads + threadIdx.x;
    if (i < n)
      atomicAdd(&h[(keys[i] >> shift) & 255], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kSortThreads)
    counts[(uint64_t)d * numTiles + blockIdx.x] = h[d];
}

/* One stable pass of an 8-bit digit over a tile of kSortTile pairs: warps rank
 * their keys per digit (match_any), the tile is put in digit order in shared
 * memory, and consecutive threads then write consecutive positions of each
 * digit's run, so the global writes coalesce. */
__global__ void __launch_bounds__(kSortThreads) digitScatter(const uint64_t *__restrict__ keys,
                                                            const uint32_t *__restrict__ vals, uint64_t n,
                                                            int shift, const uint32_t *__restrict__ offsets,
                                                            int numTiles, uint64_t *__restrict__ keysOut,
                                                            uint32_t *__restrict__ valsOut)
{
  __shared__ uint32_t wcount[kSortWarps][256];
  __shared__ uint32_t localStart[256], globalStart[256];
  __shared__ uint64_t skeys[kSortTile];
  __shared__ uint32_t svals[kSortTile];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kSortWarps * 256; i += kSortThreads)
    (&wcount[0][0])[i] = 0;
  __syncthreads();
  const uint64_t tbase = (uint64_t)blockIdx.x * kSortTile;
  const uint32_t tileN = (uint32_t)(n - tbase < (uint64_t)kSortTile ? n - tbase : (uint64_t)kSortTile);
  uint64_t wbase = tbase + (uint64_t)warp * (kSortPerLane * 32);
  uint64_t k8[kSortPerLane];
  uint32_t v8[kSortPerLane];
  uint32_t rank[kSortPerLane];
  const unsigned lt = (1u << lane) - 1;
#pragma unroll
  for (int s = 0; s < kSortPerLane; s++)
  {
    uint64_t i = wbase + (uint64_t)s * 32 + lane;
    bool ok = i < n;
    uint64_t key = ok ? keys[i] : 0;
    k8[s] = key;
    v8[s] = ok ? vals[i] : 0;
    uint32_t d = ok ? (uint32_t)((key >> shift) & 255) : 256u;
    unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t pre = (d < 256) ? wcount[warp][d] : 0;
    rank[s] = pre + __popc(peers & lt);
    __syncwarp();
    if (d < 256 && (peers & lt) == 0)
      wcount[warp][d] = pre + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit: exclusive prefix over warps, the tile's total, and where the
  // digit's run starts in the tile and in the output
  for (int d = threadIdx.x; d < 256; d += kSortThreads)
  {
    uint32_t run = 0;
    for (int w = 0; w < kSortWarps; w++)
    {
      uint32_t c = wcount[w][d];
      wcount[w][d] = run;
      run += c;
    }
    localStart[d] = run;   // the digit's count for now
    globalStart[d] = offsets[(uint64_t)d * numTiles + blockIdx.x];
  }
  __syncthreads();
  if (warp == 0)
  {
    // exclusive prefix of the 256 digit counts, 8 per lane
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
      uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
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
  for (int s = 0; s < kSortPerLane; s++)
  {
    uint64_t i = wbase + (uint64_t)s * 32 + lane;
    if (i < n)
    {
      uint32_t d = (uint32_t)((k8[s] >> shift) & 255);
      uint32_t lp = localStart[d] + wcount[warp][d] + rank[s];
      skeys[lp] = k8[s];
      svals[lp] = v8[s];
    }
  }
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < tileN; t += kSortThreads)
  {
    uint64_t key = skeys[t];
    uint32_t d = (uint32_t)((key >> shift) & 255);
    uint32_t pos = globalStart[d] + (t - localStart[d]);
    keysOut[pos] = key;
    valsOut[pos] = svals[t];
  }
}

/* Bits that differ between any key and keys[0]. */
__global__ void keySpread(const uint64_t *__restrict__ keys, uint64_t n, unsigned long long *orBits)
{
  uint64_t first = keys[0];
  uint64_t acc = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    acc |= keys[i] ^ first;
  for (int o = 16; o; o >>= 1)
    acc |= __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0 && acc)
    atomicOr(orBits, (unsigned long long)acc);
}
__global__ void pullKernel(const uint4 *__restrict__ src, uint4 *__restrict__ dst, uint64_t n16)
{
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
}  // namespace

/* Copy of a caller's host buffer into device memory, in stream order.  Pinned
 * host memory is read in place by a kernel over the CPU link (GB300: NVLink-C2C,
 * the same rate as the copy engine); anything else goes through
 * cudaMemcpyAsync. */
int wb_copy_in(wb_ctx *c, void *dst, const void *src, size_t bytes)
{
  cudaPointerAttributes at;
  const void *view = nullptr;
  if (cudaPointerGetAttributes(&at, src) == cudaSuccess)
  {
    if (at.type == cudaMemoryTypeHost && at.devicePointer)
      view = at.devicePointer;
  }
  else
    cudaGetLastError();
  if (view && bytes >= (1u << 20) && (uintptr_t)view % 16 == 0 && (uintptr_t)dst % 16 == 0)
  {
    const uint64_t n16 = bytes / 16;
    const unsigned grid = (unsigned)c->sm_count * 8;
    { pullKernel<<<grid, 256, 0, c->stream>>>((const uint4 *)view, (uint4 *)dst, n16); ++c->launches; }
    WB_CUDA(c, cudaGetLastError());
    if (bytes > n16 * 16)
      WB_CUDA(c, cudaMemcpyAsync((uint8_t *)dst + n16 * 16, (const uint8_t *)src + n16 * 16, bytes - n16 * 16,
                                 cudaMemcpyDefault, c->stream));
    return 0;
  }
  WB_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c->stream));
  return 0;
}

/* Whether kernels can dereference p: device or managed memory, or host memory
 * mapped for the device.  A pageable host pointer passed where the API wants
 * a device pointer is refused with WB_EINVAL instead of reaching a kernel. */
bool wb_device_accessible(const void *p)
{
  if (!p)
    return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess)
  {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged ||
         (at.type == cudaMemoryTypeHost && at.devicePointer == p);
}

int wb_exclusive_scan_u32(wb_ctx *c, const uint32_t *in, uint32_t *out, uint64_t n, uint32_t *total_dev)
{
  if (n == 0)
    return 0;
  uint64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1)
  {
    { scanTiles<<<1, kScanThreads, 0, c->stream>>>(in, out, n, nullptr); ++c->launches; }
  }
  else
  {
    // block sums live in a scratch region carved per recursion level
    uint64_t need = 0;
    for (uint64_t t = tiles; t > 1; t = (t + kScanTile - 1) / kScanTile)
      need += 2 * t;
    int rc = wb_ensure(c, c->scanTmp, (need + 64) * sizeof(uint32_t));
    if (rc)
      return rc;
    uint32_t *sums = (uint32_t *)c->scanTmp.p;
    uint32_t *sumsEx = sums + tiles;
    { scanTiles<<<(unsigned)tiles, kScanThreads, 0, c->stream>>>(in, out, n, sums); ++c->launches; }
    // recurse on the block sums (their scratch follows)
    DevBuf saved = c->scanTmp;
    // shift scratch window for the nested call
    c->scanTmp.p = (void *)(sumsEx + tiles);
    c->scanTmp.cap = saved.cap - 2 * tiles * sizeof(uint32_t);
    rc = wb_exclusive_scan_u32(c, sums, sumsEx, tiles, nullptr);
    c->scanTmp = saved;
    if (rc)
      return rc;
    { addOffsets<<<(unsigned)tiles, kScanThreads, 0, c->stream>>>(out, n, sumsEx); ++c->launches; }
  }
  if (total_dev)
    { totalOf<<<1, 1, 0, c->stream>>>(in, out, n, total_dev); ++c->launches; }
  WB_CUDA(c, cudaGetLastError());
  return 0;
}

int wb_radix_sort_pairs(wb_ctx *c, uint64_t *&keys, uint32_t *&vals, uint64_t *keysAlt, uint32_t *valsAlt,
                        uint64_t n, int beginBit, int endBit)
{
  if (n <= 1)
    return 0;
  int rc = wb_ensure(c, c->small, 4096);
  if (rc)
    return rc;
  unsigned long long *dOr = (unsigned long long *)c->small.p;
  WB_CUDA(c, cudaMemsetAsync(dOr, 0, 8, c->stream));
  { keySpread<<<c->sm_count * 4, 256, 0, c->stream>>>(keys, n, dOr); ++c->launches; }
  unsigned long long spread = 0;
  WB_CUDA(c, cudaMemcpyAsync(&spread, dOr, 8, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  int numTiles = (int)((n + kSortTile - 1) / kSortTile);
  size_t cntBytes = (size_t)numTiles * 256 * sizeof(uint32_t);
  rc = wb_ensure(c, c->tmp32b, 2 * cntBytes + 64);
  if (rc)
    return rc;
  uint32_t *counts = (uint32_t *)c->tmp32b.p;
  uint32_t *offs = counts + (size_t)numTiles * 256;
  for (int shift = beginBit; shift < endBit; shift += 8)
  {
    uint64_t mask = (shift + 8 >= 64) ? (~0ULL << shift) : (((1ULL << 8) - 1) << shift);
    if ((spread & mask) == 0)
      continue;   // digit identical for all keys: pass would be the identity
    { digitCounts<<<numTiles, kSortThreads, 0, c->stream>>>(keys, n, shift, counts, numTiles); ++c->launches; }
    rc = wb_exclusive_scan_u32(c, counts, offs, (uint64_t)numTiles * 256, nullptr);
    if (rc)
      return rc;
    { digitScatter<<<numTiles, kSortThreads, 0, c->stream>>>(keys, vals, n, shift, offs, numTiles, keysAlt, valsAlt); ++c->launches; }
    WB_CUDA(c, cudaGetLastError());
    uint64_t *tk = keys;
    keys = keysAlt;
    keysAlt = tk;
    uint32_t *tv = vals;
    vals = valsAlt;
    valsAlt = tv;
  }
  return 0;
}

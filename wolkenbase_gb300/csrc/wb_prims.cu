/* Device-wide primitives written for this library: exclusive scan of u32 and
 * a stable LSD radix sort of (u64 key, u32 value) pairs (one sweep per 8-bit
 * digit, see below).
 */
#include <cuda_runtime.h>
#include <algorithm>
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

/* ---------------- radix sort ----------------
 * One sweep per 8-bit digit (the decoupled look-back scheme of Merrill and
 * Garland's single-pass scan, applied per digit as in Adinets and Merrill's
 * "Onesweep" radix sort).  One kernel histograms every digit position of the
 * keys at once; the exclusive scans give each digit value's first output
 * slot per pass.  Each pass is then one kernel: a CTA takes the next tile of
 * kOsTile pairs in launch order (an atomic ticket), ranks its keys per digit
 * (warps walk their keys in order with match_any, so the sort is stable),
 * publishes its per-digit counts, looks back over the tiles before it for
 * their per-digit prefixes, and scatters its keys in digit order through
 * shared memory, so each digit's run is written contiguously.  A digit
 * position whose keys all share one value is skipped.  Every look-back wait
 * is bounded: a wait that runs out sets an error word and the sort reports
 * WB_ETIMEDOUT instead of hanging. */
constexpr int kOsThreads = 256;
constexpr int kOsWarps = kOsThreads / 32;
constexpr int kOsPerLane = 12;
constexpr int kOsTile = kOsThreads * kOsPerLane;   // 3072 pairs per tile
constexpr unsigned long long kOsAgg = 1ull << 62, kOsPre = 2ull << 62, kOsVal = (1ull << 62) - 1;
constexpr long long kOsSpinLimit = 1ll << 22;

/* Counts of every 8-bit digit value at every digit position: hist[p][v]. */
__global__ void __launch_bounds__(256) osHistogram(const uint64_t *__restrict__ keys, uint64_t n,
                                                   uint32_t *__restrict__ hist)
{
  __shared__ uint32_t h[8][256];
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x)
    (&h[0][0])[i] = 0;
  __syncthreads();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
  {
    const uint64_t k = keys[i];
#pragma unroll
    for (int p = 0; p < 8; p++)
      atomicAdd(&h[p][(k >> (8 * p)) & 255], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x)
  {
    const uint32_t v = (&h[0][0])[i];
    if (v)
      atomicAdd(&hist[i], v);
  }
}

/* base[p][v] = exclusive prefix of hist[p][.] at v; block p, 256 threads. */
__global__ void __launch_bounds__(256) osBases(const uint32_t *__restrict__ hist, uint32_t *__restrict__ base)
{
  __shared__ uint32_t w[8];
  const int p = blockIdx.x, v = threadIdx.x, lane = v & 31, warp = v >> 5;
  const uint32_t x = hist[p * 256 + v];
  const uint32_t inc = warpInclusive(x);
  if (lane == 31)
    w[warp] = inc;
  __syncthreads();
  uint32_t off = 0;
  for (int k = 0; k < warp; k++)
    off += w[k];
  base[p * 256 + v] = off + inc - x;
}

__global__ void __launch_bounds__(kOsThreads) osPass(const uint64_t *__restrict__ keys,
                                                     const uint32_t *__restrict__ vals, uint64_t n, int shift,
                                                     const uint32_t *__restrict__ base,
                                                     unsigned long long *__restrict__ status,
                                                     uint32_t *__restrict__ ticket, int *__restrict__ err,
                                                     uint64_t *__restrict__ keysOut, uint32_t *__restrict__ valsOut)
{
  __shared__ uint32_t wcount[kOsWarps][256];
  __shared__ uint32_t localStart[256], globalStart[256];
  __shared__ uint64_t skeys[kOsTile];
  __shared__ uint32_t svals[kOsTile];
  __shared__ uint32_t sTile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0)
    sTile = atomicAdd(ticket, 1u);
  for (int i = threadIdx.x; i < kOsWarps * 256; i += kOsThreads)
    (&wcount[0][0])[i] = 0;
  __syncthreads();
  const uint64_t tile = sTile;
  const uint64_t tbase = tile * kOsTile;
  const uint32_t tileN = (uint32_t)(n - tbase < (uint64_t)kOsTile ? n - tbase : (uint64_t)kOsTile);
  const uint64_t wbase = tbase + (uint64_t)warp * (kOsPerLane * 32);
  uint64_t kk[kOsPerLane];
  uint32_t vv[kOsPerLane];
  uint32_t rank[kOsPerLane];
  const unsigned lt = (1u << lane) - 1;
#pragma unroll
  for (int q = 0; q < kOsPerLane; q++)
  {
    const uint64_t i = wbase + (uint64_t)q * 32 + lane;
    const bool ok = i < n;
    kk[q] = ok ? keys[i] : 0;
    vv[q] = ok ? vals[i] : 0;
  }
#pragma unroll
  for (int q = 0; q < kOsPerLane; q++)
  {
    const uint64_t i = wbase + (uint64_t)q * 32 + lane;
    const uint32_t d = i < n ? (uint32_t)((kk[q] >> shift) & 255) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t pre = d < 256 ? wcount[warp][d] : 0;
    rank[q] = pre + __popc(peers & lt);
    __syncwarp();
    if (d < 256 && (peers & lt) == 0)
      wcount[warp][d] = pre + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    // thread d: the digit's exclusive prefix over warps, its count in the
    // tile, publication, and the look-back over earlier tiles
    const int d = threadIdx.x;
    uint32_t run = 0;
    for (int w = 0; w < kOsWarps; w++)
    {
      const uint32_t c = wcount[w][d];
      wcount[w][d] = run;
      run += c;
    }
    localStart[d] = run;
    unsigned long long *mine = status + tile * 256 + d;
    unsigned long long excl = 0;
    if (tile == 0)
      atomicExch(mine, kOsPre | (unsigned long long)run);
    else
    {
      atomicExch(mine, kOsAgg | (unsigned long long)run);
      for (long long p = (long long)tile - 1; p >= 0; p--)
      {
        const volatile unsigned long long *sp = status + (uint64_t)p * 256 + d;
        unsigned long long v = *sp;
        long long spins = 0;
        while ((v >> 62) == 0)
        {
          if (++spins > kOsSpinLimit)
          {
            atomicExch(err, 1);
            v = kOsPre;
            break;
          }
          __nanosleep(32);
          v = *sp;
        }
        excl += v & kOsVal;
        if ((v >> 62) == 2)
          break;
      }
      atomicExch(mine, kOsPre | (excl + run));
    }
    globalStart[d] = base[d] + (uint32_t)excl;
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
    const uint32_t inc = warpInclusive(sum);
    uint32_t r = inc - sum;
#pragma unroll
    for (int q = 0; q < 8; q++)
    {
      localStart[lane * 8 + q] = r;
      r += c[q];
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < kOsPerLane; q++)
  {
    const uint64_t i = wbase + (uint64_t)q * 32 + lane;
    if (i < n)
    {
      const uint32_t d = (uint32_t)((kk[q] >> shift) & 255);
      const uint32_t lp = localStart[d] + wcount[warp][d] + rank[q];
      skeys[lp] = kk[q];
      svals[lp] = vv[q];
    }
  }
  __syncthreads();
  for (uint32_t t = threadIdx.x; t < tileN; t += kOsThreads)
  {
    const uint64_t key = skeys[t];
    const uint32_t d = (uint32_t)((key >> shift) & 255);
    const uint64_t pos = (uint64_t)globalStart[d] + (t - localStart[d]);
    keysOut[pos] = key;
    valsOut[pos] = svals[t];
  }
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
  if (n > 0xffffffffull)
    return wb_fail(c, WB_EINVAL, "radix sort: more than 2^32-1 pairs");
  // aux words: histograms [0, 2048), bases [2048, 4096), tickets [4096, 4104), error at 4104
  int rc = wb_ensure(c, c->sortAux, (4096 + 64) * 4);
  if (rc)
    return rc;
  uint32_t *aux = (uint32_t *)c->sortAux.p;
  uint32_t *hist = aux, *base = aux + 2048, *tickets = aux + 4096;
  int *err = (int *)(aux + 4104);
  const uint64_t numTiles = (n + kOsTile - 1) / kOsTile;
  if ((rc = wb_ensure(c, c->tmp32b, numTiles * 256 * 8 + 64)))
    return rc;
  unsigned long long *status = (unsigned long long *)c->tmp32b.p;
  WB_CUDA(c, cudaMemsetAsync(aux, 0, (4096 + 64) * 4, c->stream));
  { osHistogram<<<(unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)c->sm_count * 8), 256, 0, c->stream>>>(
        keys, n, hist); ++c->launches; }
  { osBases<<<8, 256, 0, c->stream>>>(hist, base); ++c->launches; }
  uint32_t h[2048];
  WB_CUDA(c, cudaMemcpyAsync(h, hist, sizeof h, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  for (int shift = beginBit; shift < endBit && shift < 64; shift += 8)
  {
    const int p = shift / 8;
    bool constant = false;
    for (int v = 0; v < 256 && !constant; v++)
      constant = h[p * 256 + v] == n;
    if (constant)
      continue;   // every key has the same digit here: the pass would be the identity
    WB_CUDA(c, cudaMemsetAsync(status, 0, numTiles * 256 * 8, c->stream));
    { osPass<<<(unsigned)numTiles, kOsThreads, 0, c->stream>>>(keys, vals, n, shift, base + p * 256, status,
                                                               tickets + p, err, keysAlt, valsAlt); ++c->launches; }
    WB_CUDA(c, cudaGetLastError());
    uint64_t *tk = keys;
    keys = keysAlt;
    keysAlt = tk;
    uint32_t *tv = vals;
    vals = valsAlt;
    valsAlt = tv;
  }
  int e = 0;
  WB_CUDA(c, cudaMemcpyAsync(&e, err, 4, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  if (e)
    return wb_fail(c, WB_ETIMEDOUT, "radix sort: a look-back wait ran out");
  return 0;
}

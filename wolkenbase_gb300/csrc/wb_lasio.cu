/* LAS point records either side of the path: every field of a record as
 * LasHeader::readPoint decodes it, and the class-split writer -- CloudOutput's
 * openFiles / writeFiles / closeFiles with LasHeader::setScale, writePoint and
 * writeHeader.
 *
 *  wb_las_decode           readPoint (las.cpp:735-820) for every record, one
 *                          array per LasPoint field
 *  wb_las_write_output     openFiles + writeFiles (cloudoutput.cpp:116-231):
 *                          the files of each class, balanced over the octree
 *                          blocks by points_per_file, every record re-encoded
 *                          by writePoint (las.cpp:822-904) on the device with
 *                          the header figures writePoint accumulates
 *  wb_las_header_bytes     writeHeader (las.cpp:540-595)
 *  wb_las_file_name        the names openFiles gives (cloudoutput.cpp:27-185)
 *  wb_las_write_files      all of it, the files on disk (closeFiles, 232-245)
 *  wb_las_join_point_format, wb_las_combine_scales
 *                          joinPointFormat (las.cpp:103-118); combineScales,
 *                          combine1Scale (las.cpp:906-944) and manygcd
 *                          (manygcd.cpp:28-74)
 *
 * On the device a record is read once into a per-thread slot of shared memory
 * (word loads where the stride allows), parsed there, and the re-encoded record
 * is stored to its place in its file.  The writer runs one warp per octree
 * block: the block's points are ranked within their class with warp match and
 * popcount, so the one serial step -- choosing each block's file when a class
 * spans several files -- is a heap walk over the (block, class) counts on the
 * host.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <functional>
#include <queue>
#include <string>
#include <vector>
#include "wb_internal.h"

namespace
{
constexpr int kMaskGps = 0x7fa, kMaskRgb = 0x5ac, kMaskNir = 0x500, kMaskWave = 0x630;   // las.cpp:34-37
constexpr int kSlotWords = 17;   // 68 bytes: the longest record (67, format 10) in whole words
constexpr int kBlock = 256;
constexpr int kSharedFiles = 64; // files whose header figures a block gathers in shared memory

/* Where the optional parts of a record of format f start (-1: absent) and its
 * length, in the order readPoint reads them (las.cpp:776-806). */
struct Layout
{
  int len, gps, rgb, nir, wave;
};

__host__ __device__ inline Layout layoutOf(int f)
{
  Layout L;
  int o = f < 6 ? 20 : 22;
  L.gps = L.rgb = L.nir = L.wave = -1;
  if ((1 << f) & kMaskGps)
  {
    L.gps = o;
    o += 8;
  }
  if ((1 << f) & kMaskRgb)
  {
    L.rgb = o;
    o += 6;
  }
  if ((1 << f) & kMaskNir)
  {
    L.nir = o;
    o += 2;
  }
  if ((1 << f) & kMaskWave)
  {
    L.wave = o;
    o += 29;
  }
  L.len = o;
  return L;
}

/* A LasPoint in registers. */
struct LasPt
{
  int32_t X[3];        /* the record integers */
  double gps;
  int32_t angle;
  uint32_t angleRaw;   /* the record's scan-angle byte or short */
  uint16_t intensity, ret, nret, cls, flags, chan, user, src, r, g, b, nir;
  bool sdir, edge;
};

struct Decode
{
  double off[3], scale[3], unit;
};

__device__ __forceinline__ uint32_t rd16(const uint8_t *s, int o)
{
  return (uint32_t)s[o] | ((uint32_t)s[o + 1] << 8);
}
__device__ __forceinline__ uint32_t rd32(const uint8_t *s, int o)
{
  return rd16(s, o) | (rd16(s, o + 2) << 16);
}
__device__ __forceinline__ uint64_t rd64(const uint8_t *s, int o)
{
  return (uint64_t)rd32(s, o) | ((uint64_t)rd32(s, o + 4) << 32);
}
__device__ __forceinline__ void wr16(uint8_t *s, int o, uint32_t v)
{
  s[o] = (uint8_t)v;
  s[o + 1] = (uint8_t)(v >> 8);
}
__device__ __forceinline__ void wr32(uint8_t *s, int o, uint32_t v)
{
  wr16(s, o, v);
  wr16(s, o + 2, v >> 16);
}
__device__ __forceinline__ void wr64(uint8_t *s, int o, uint64_t v)
{
  wr32(s, o, (uint32_t)v);
  wr32(s, o + 4, (uint32_t)(v >> 32));
}

/* lrint of a double and the C conversion of the long to a narrower integer
 * (two's complement wrap): the reference's (int)lrint(...), put(...) and
 * writeleshort(...) of a long. */
__device__ __forceinline__ uint64_t lrintBits(double v)
{
  return (uint64_t)__double2ll_rn(v);
}

/* Scan angles.  A record holds a signed byte of degrees (formats 0-5) or a
 * signed short of 0.006 degrees (6-10); readPoint turns it into 2^31 units
 * per turn with degtobin, and writePoint back with lrint(bintodeg(...)) or
 * lrint(bintodeg(...)/0.006) (angle.cpp:199-243, las.cpp:758, 772, 857, 866).
 * Both are functions of the record's value alone, so they are tabulated once
 * per context on the host (double arithmetic as the reference's, no FMA) and
 * the kernels look them up instead of running FP64 divisions. */
struct AngleTabs
{
  const int32_t *bin8, *bin16;      /* degtobin of each byte / short value   */
  const uint8_t *deg8of8, *deg8of16; /* written byte (formats 0-5) of each value */
  const uint16_t *deg16of8, *deg16of16; /* written short (formats 6-10) of each value */
};

constexpr size_t kAngleBytes = 256 * 4 + 65536 * 4 + 256 + 65536 + 256 * 2 + 65536 * 2;

int32_t hostDegToBin(double deg)
{
  double ip;
  double f = 2 * modf(deg / 360 / 2, &ip);
  if (f >= 1)
    f -= 2;
  if (f < -1)
    f += 2;
  return (int32_t)(uint32_t)(uint64_t)(int64_t)llrint(2147483648. * f);
}

double hostBinToDeg(int32_t a)
{
  return a / 2147483648. * 360;
}

/* Builds (once per context) and returns the device tables. */
int angleTables(wb_ctx *c, AngleTabs &t)
{
  const bool ready = c->lasAngles.p && c->lasAngles.cap >= kAngleBytes;
  int rc = wb_ensure(c, c->lasAngles, kAngleBytes);
  if (rc)
    return rc;
  uint8_t *base = (uint8_t *)c->lasAngles.p;
  t.bin8 = (const int32_t *)base;
  t.bin16 = t.bin8 + 256;
  t.deg16of8 = (const uint16_t *)(t.bin16 + 65536);
  t.deg16of16 = t.deg16of8 + 256;
  t.deg8of8 = (const uint8_t *)(t.deg16of16 + 65536);
  t.deg8of16 = t.deg8of8 + 256;
  if (ready)
    return 0;
  std::vector<uint8_t> h(kAngleBytes);
  int32_t *bin8 = (int32_t *)h.data(), *bin16 = bin8 + 256;
  uint16_t *d16of8 = (uint16_t *)(bin16 + 65536), *d16of16 = d16of8 + 256;
  uint8_t *d8of8 = (uint8_t *)(d16of16 + 65536), *d8of16 = d8of8 + 256;
  for (int v = 0; v < 256; v++)
    bin8[v] = hostDegToBin((double)(int8_t)v);
  for (int v = 0; v < 65536; v++)
    bin16[v] = hostDegToBin((double)(int16_t)v * 0.006);
  for (int v = 0; v < 256; v++)
  {
    d8of8[v] = (uint8_t)llrint(hostBinToDeg(bin8[v]));
    d16of8[v] = (uint16_t)llrint(hostBinToDeg(bin8[v]) / 0.006);
  }
  for (int v = 0; v < 65536; v++)
  {
    d8of16[v] = (uint8_t)llrint(hostBinToDeg(bin16[v]));
    d16of16[v] = (uint16_t)llrint(hostBinToDeg(bin16[v]) / 0.006);
  }
  WB_CUDA(c, cudaMemcpyAsync(base, h.data(), kAngleBytes, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));
  return 0;
}

/* Copies the first len bytes of a record into a shared-memory slot; words
 * when the record start and stride are 4-byte aligned (then the stride holds
 * len rounded up to a word). */
__device__ __forceinline__ void loadRecord(uint8_t *slot, const uint8_t *src, int len, bool words)
{
  if (words)
  {
    const uint32_t *w = (const uint32_t *)src;
    uint32_t *d = (uint32_t *)slot;
    for (int k = 0; k < (len + 3) >> 2; k++)
      d[k] = __ldg(w + k);
  }
  else
    for (int k = 0; k < len; k++)
      slot[k] = __ldg(src + k);
}

__device__ __forceinline__ void storeRecord(uint8_t *dst, const uint8_t *slot, int len, int width)
{
  if (width == 4)
    for (int k = 0; k < len >> 2; k++)
      ((uint32_t *)dst)[k] = ((const uint32_t *)slot)[k];
  else if (width == 2)
    for (int k = 0; k < len >> 1; k++)
      ((uint16_t *)dst)[k] = ((const uint16_t *)slot)[k];
  else
    for (int k = 0; k < len; k++)
      dst[k] = slot[k];
}

/* LasHeader::readPoint (las.cpp:735-820) from a record in shared memory. */
__device__ __forceinline__ void parseRecord(const uint8_t *s, int f, const Layout &L, const Decode &d,
                                            const AngleTabs &at, LasPt &p)
{
  p.X[0] = (int32_t)rd32(s, 0);
  p.X[1] = (int32_t)rd32(s, 4);
  p.X[2] = (int32_t)rd32(s, 8);
  p.intensity = (uint16_t)rd16(s, 12);
  if (f < 6)
  {
    const uint32_t t = s[14], c = s[15];
    p.ret = t & 7;
    p.nret = (t >> 3) & 7;
    p.sdir = (t >> 6) & 1;
    p.edge = (t >> 7) & 1;
    p.flags = (c >> 5) & 7;
    p.cls = c & 31;
    p.chan = 0;
    p.angleRaw = s[16];
    p.angle = __ldg(at.bin8 + p.angleRaw);
    p.user = s[17];
    p.src = (uint16_t)rd16(s, 18);
  }
  else
  {
    const uint32_t t = s[14], u = s[15];
    p.ret = t & 15;
    p.nret = (t >> 4) & 15;
    p.flags = u & 15;
    p.chan = (u >> 4) & 3;
    p.sdir = (u >> 6) & 1;
    p.edge = (u >> 7) & 1;
    p.cls = s[16];
    p.user = s[17];
    p.angleRaw = rd16(s, 18);
    p.angle = __ldg(at.bin16 + p.angleRaw);
    p.src = (uint16_t)rd16(s, 20);
  }
  p.gps = L.gps >= 0 ? __longlong_as_double((long long)rd64(s, L.gps)) : 0.0;
  if (L.rgb >= 0)
  {
    p.r = (uint16_t)rd16(s, L.rgb);
    p.g = (uint16_t)rd16(s, L.rgb + 2);
    p.b = (uint16_t)rd16(s, L.rgb + 4);
  }
  else
    p.r = p.g = p.b = 0;
  p.nir = L.nir >= 0 ? (uint16_t)rd16(s, L.nir) : 0;
}

/* The location readPoint computes (las.cpp:808): (offset + scale*X) * unit. */
__device__ __forceinline__ double decodeAxis(const Decode &d, int32_t X, int k)
{
  const double v = d.off[k] + d.scale[k] * (double)X;
  return d.unit != 1 ? v * d.unit : v;   // x * 1 == x
}

struct Encode
{
  double off[3], scale[3], inv[3], unit;   /* inv = 1/scale rounded */
  bool shift[3];                           /* the record integer moves by a constant */
  long long by[3];
};

/* The record integer writePoint computes (las.cpp:827-829):
 * lrint((v/unit - off)/scale), wrapped to int.  The quotient is first taken
 * as a product with the rounded reciprocal, which lies within 3 units in the
 * last place of the rounded quotient; unless that puts it within 2^-19 of a
 * half-integer (or outside the int range), both round to the same integer, so
 * the FP64 division runs only in those rare cases. */
__device__ __forceinline__ int32_t quantise(double v, const Encode &e, int k)
{
  if (e.unit != 1)   // v / 1 == v
    v = v / e.unit;
  const double t = v - e.off[k];
  const double y = t * e.inv[k];
  const double r = rint(y);
  if (fabs(y) < 2147483648.0 && 0.5 - fabs(y - r) > 0x1p-19)
    return (int32_t)(long long)r;
  return (int32_t)(uint32_t)lrintBits(t / e.scale[k]);
}

/* LasHeader::writePoint (las.cpp:822-904) into a shared-memory slot; the
 * waveform part is written as zeros (the reference's build without WAVEFORM). */
__device__ __forceinline__ void encodeRecord(uint8_t *o, int f, const Layout &L, const LasPt &p, const int32_t *q,
                                             bool in16, const AngleTabs &t)
{
  wr32(o, 0, (uint32_t)q[0]);
  wr32(o, 4, (uint32_t)q[1]);
  wr32(o, 8, (uint32_t)q[2]);
  wr16(o, 12, p.intensity);
  if (f < 6)
  {
    o[14] = (uint8_t)((p.ret & 7) + ((p.nret & 7) << 3) + ((p.sdir & 1) << 6) + ((p.edge & 1) << 7));
    o[15] = (uint8_t)((p.cls & 31) + ((p.flags & 7) << 5));
    o[16] = __ldg((in16 ? t.deg8of16 : t.deg8of8) + p.angleRaw);
    o[17] = (uint8_t)p.user;
    wr16(o, 18, p.src);
  }
  else
  {
    o[14] = (uint8_t)((p.ret & 15) + ((p.nret & 15) << 4));
    o[15] = (uint8_t)((p.flags & 15) + ((p.chan & 3) << 4) + ((p.sdir & 1) << 6) + ((p.edge & 1) << 7));
    o[16] = (uint8_t)p.cls;
    o[17] = (uint8_t)p.user;
    wr16(o, 18, __ldg((in16 ? t.deg16of16 : t.deg16of8) + p.angleRaw));
    wr16(o, 20, p.src);
  }
  if (L.gps >= 0)
    wr64(o, L.gps, (uint64_t)__double_as_longlong(p.gps));
  if (L.rgb >= 0)
  {
    wr16(o, L.rgb, p.r);
    wr16(o, L.rgb + 2, p.g);
    wr16(o, L.rgb + 4, p.b);
  }
  if (L.nir >= 0)
    wr16(o, L.nir, p.nir);
  if (L.wave >= 0)
    for (int k = 0; k < 29; k++)
      o[L.wave + k] = 0;
}

/* ---- wb_las_decode ---- */

struct DecodeArgs
{
  const uint8_t *rec;
  uint64_t n;
  uint32_t stride;
  int fmt;
  bool words, vec16;
  Decode d;
  AngleTabs t;
  wb_las_points o;
};

/* One warp per 32 consecutive records: when the records start on a 16-byte
 * boundary and a record is at most kStageStride bytes, the warp copies its 32
 * records into shared memory with coalesced 16-byte loads and each lane parses
 * its own record there; otherwise each lane loads its record into its slot. */
constexpr int kStageStride = 80;

__global__ void __launch_bounds__(kBlock) decodeKernel(const DecodeArgs a)
{
  __shared__ __align__(16) uint8_t stage[kBlock / 32][32 * kStageStride];
  __shared__ uint32_t slots[kBlock * kSlotWords];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const Layout L = layoutOf(a.fmt);
  const bool staged = a.vec16 && a.stride <= (uint32_t)kStageStride;
  const uint64_t chunks = (a.n + 31) / 32;
  for (uint64_t ch = (uint64_t)blockIdx.x * (kBlock / 32) + warp; ch < chunks; ch += (uint64_t)gridDim.x * (kBlock / 32))
  {
    const uint64_t i0 = ch * 32, i = i0 + lane;
    const uint8_t *s;
    if (staged)
    {
      // 32 records of a multiple-of-32 stride start on a 16-byte boundary
      const uint64_t start = i0 * a.stride;
      const uint32_t bytes = (uint32_t)((min(i0 + 32, a.n) - i0) * a.stride);
      const uint4 *src = (const uint4 *)(a.rec + start);
      uint4 *dst = (uint4 *)stage[warp];
      const uint32_t vecs = bytes >> 4;
      for (uint32_t v = lane; v < vecs; v += 32)
        dst[v] = __ldg(src + v);
      for (uint32_t b = (vecs << 4) + lane; b < bytes; b += 32)
        stage[warp][b] = __ldg(a.rec + start + b);
      __syncwarp();
      s = stage[warp] + lane * a.stride;
    }
    else
    {
      uint8_t *slot = (uint8_t *)(slots + threadIdx.x * kSlotWords);
      if (i < a.n)
        loadRecord(slot, a.rec + i * a.stride, L.len, a.words);
      s = slot;
    }
    if (i < a.n)
    {
      LasPt p;
      parseRecord(s, a.fmt, L, a.d, a.t, p);
      const wb_las_points &o = a.o;
      if (o.x) o.x[i] = decodeAxis(a.d, p.X[0], 0);
      if (o.y) o.y[i] = decodeAxis(a.d, p.X[1], 1);
      if (o.z) o.z[i] = decodeAxis(a.d, p.X[2], 2);
      if (o.intensity) o.intensity[i] = p.intensity;
      if (o.return_num) o.return_num[i] = p.ret;
      if (o.n_returns) o.n_returns[i] = p.nret;
      if (o.scan_direction) o.scan_direction[i] = p.sdir;
      if (o.edge_line) o.edge_line[i] = p.edge;
      if (o.classification) o.classification[i] = p.cls;
      if (o.class_flags) o.class_flags[i] = p.flags;
      if (o.scanner_channel) o.scanner_channel[i] = p.chan;
      if (o.user_data) o.user_data[i] = p.user;
      if (o.scan_angle) o.scan_angle[i] = p.angle;
      if (o.point_source) o.point_source[i] = p.src;
      if (o.gps_time) o.gps_time[i] = p.gps;
      if (o.red) o.red[i] = p.r;
      if (o.green) o.green[i] = p.g;
      if (o.blue) o.blue[i] = p.b;
      if (o.nir) o.nir[i] = p.nir;
    }
    __syncwarp();
  }
}

/* ---- wb_las_write_output ---- */

/* Header figures of one output file while it is written (las.cpp:832-845,
 * 900-902): extreme record integers (decoding is monotone in them) and the
 * point counts, [0] all and [r] of return number r. */
struct FileStat
{
  int32_t mn[3], mx[3];
  unsigned long long cnt[16];
};

struct WriteArgs
{
  const uint8_t *rec;
  uint32_t stride;
  int inFmt, outFmt;
  bool inWords;
  int outWidth;                  /* widest store the output records allow: 4, 2 or 1 */
  Decode d;
  Encode e;
  AngleTabs t;
  uint8_t *out;
  uint64_t nLeaves;
  const uint32_t *leafFirst, *leafCount, *sidx;
  const uint8_t *cls;            /* class byte per stored point, in store order */
  uint32_t nSets;
  uint16_t setOf[256];           /* class byte -> set of files */
  unsigned long long *base;      /* per (block, set): next output record */
  const uint32_t *fileOf;        /* per (block, set): the file chosen */
  uint32_t nFiles;
  FileStat *stats;
};

/* Stored points per (block, set): one warp per block. */
__global__ void __launch_bounds__(kBlock) setCountKernel(const WriteArgs a, uint32_t *__restrict__ counts)
{
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t leaf = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); leaf < a.nLeaves; leaf += warps)
  {
    const uint32_t first = a.leafFirst[leaf], cnt = a.leafCount[leaf];
    for (uint32_t c0 = 0; c0 < cnt; c0 += 32)
    {
      const bool valid = c0 + lane < cnt;
      const unsigned act = __ballot_sync(0xffffffffu, valid);
      if (valid)
      {
        const uint32_t s = a.setOf[a.cls[first + c0 + lane]];
        const unsigned gm = __match_any_sync(act, s);
        if (lane == __ffs(gm) - 1)
          counts[leaf * a.nSets + s] += __popc(gm);
      }
      __syncwarp();
    }
  }
}

template <bool SHARED_STATS>
__global__ void __launch_bounds__(kBlock) writeKernel(const WriteArgs a)
{
  extern __shared__ uint4 dyn[];
  uint32_t *inSlots = (uint32_t *)dyn;
  uint32_t *outSlots = inSlots + kBlock * kSlotWords;
  FileStat *sst = (FileStat *)(outSlots + kBlock * kSlotWords);
  FileStat *st = SHARED_STATS ? sst : a.stats;
  if (SHARED_STATS)
  {
    for (uint32_t f = threadIdx.x; f < a.nFiles; f += blockDim.x)
    {
      for (int k = 0; k < 3; k++)
      {
        sst[f].mn[k] = INT32_MAX;
        sst[f].mx[k] = INT32_MIN;
      }
      for (int k = 0; k < 16; k++)
        sst[f].cnt[k] = 0;
    }
    __syncthreads();
  }
  uint8_t *si = (uint8_t *)(inSlots + threadIdx.x * kSlotWords);
  uint8_t *so = (uint8_t *)(outSlots + threadIdx.x * kSlotWords);
  const Layout Li = layoutOf(a.inFmt), Lo = layoutOf(a.outFmt);
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1;
  const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
  for (uint64_t leaf = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); leaf < a.nLeaves; leaf += warps)
  {
    const uint32_t first = a.leafFirst[leaf], cnt = a.leafCount[leaf];
    for (uint32_t c0 = 0; c0 < cnt; c0 += 32)
    {
      const bool valid = c0 + lane < cnt;
      const unsigned act = __ballot_sync(0xffffffffu, valid);
      if (valid)
      {
        const uint32_t idx = a.sidx[first + c0 + lane];
        const uint8_t cl = a.cls[first + c0 + lane];
        const uint32_t s = a.setOf[cl];
        loadRecord(si, a.rec + (uint64_t)idx * a.stride, Li.len, a.inWords);
        LasPt p;
        parseRecord(si, a.inFmt, Li, a.d, a.t, p);
        p.cls = cl;
        int32_t q[3];
        for (int k = 0; k < 3; k++)
          q[k] = a.e.shift[k] ? (int32_t)(uint32_t)(unsigned long long)((long long)p.X[k] + a.e.by[k])
                              : quantise(decodeAxis(a.d, p.X[k], k), a.e, k);
        encodeRecord(so, a.outFmt, Lo, p, q, a.inFmt >= 6, a.t);
        // the block's points of one set go to one file, in store order
        const unsigned gm = __match_any_sync(act, s);
        const int leader = __ffs(gm) - 1;
        unsigned long long b = 0;
        uint32_t file = 0;
        if (lane == leader)
        {
          b = atomicAdd(&a.base[leaf * a.nSets + s], (unsigned long long)__popc(gm));
          file = a.fileOf[leaf * a.nSets + s];
        }
        b = __shfl_sync(act, b, leader);
        file = __shfl_sync(act, file, leader);
        storeRecord(a.out + (b + __popc(gm & lt)) * (uint64_t)Lo.len, so, Lo.len, a.outWidth);
        int32_t mn[3], mx[3];
        for (int k = 0; k < 3; k++)
        {
          mn[k] = __reduce_min_sync(gm, q[k]);
          mx[k] = __reduce_max_sync(gm, q[k]);
        }
        if (lane == leader)
        {
          for (int k = 0; k < 3; k++)
          {
            atomicMin(&st[file].mn[k], mn[k]);
            atomicMax(&st[file].mx[k], mx[k]);
          }
          atomicAdd(&st[file].cnt[0], (unsigned long long)__popc(gm));
        }
        // nPoints[returnNum] for return numbers 1-15 (las.cpp:900-901)
        const unsigned rm = __match_any_sync(act, (s << 4) | (p.ret & 15));
        if (p.ret > 0 && p.ret < 16 && lane == __ffs(rm) - 1)
          atomicAdd(&st[file].cnt[p.ret], (unsigned long long)__popc(rm));
      }
      __syncwarp();
    }
  }
  if (SHARED_STATS)
  {
    __syncthreads();
    for (uint32_t f = threadIdx.x; f < a.nFiles; f += blockDim.x)
    {
      if (!sst[f].cnt[0])
        continue;
      for (int k = 0; k < 3; k++)
      {
        atomicMin(&a.stats[f].mn[k], sst[f].mn[k]);
        atomicMax(&a.stats[f].mx[k], sst[f].mx[k]);
      }
      for (int k = 0; k < 16; k++)
        if (sst[f].cnt[k])
          atomicAdd(&a.stats[f].cnt[k], sst[f].cnt[k]);
    }
  }
}

__global__ void statInit(FileStat *st, uint32_t n)
{
  for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x)
  {
    for (int k = 0; k < 3; k++)
    {
      st[f].mn[k] = INT32_MAX;
      st[f].mx[k] = INT32_MIN;
    }
    for (int k = 0; k < 16; k++)
      st[f].cnt[k] = 0;
  }
}

/* The class byte of every stored point in store order: from the last
 * classify's store-order labels where a tile decided the point (sequential
 * reads), else from the per-record class bytes (recCls). */
__global__ void storeClassKernel(uint64_t nd, const uint32_t *__restrict__ sidx, const int32_t *__restrict__ owner,
                                 const uint8_t *__restrict__ label, const uint8_t *__restrict__ recCls,
                                 uint8_t *__restrict__ out)
{
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nd; j += (uint64_t)gridDim.x * blockDim.x)
    out[j] = (owner && owner[j] >= 0) ? label[j] : recCls[sidx[j]];
}

__global__ void storedTotals(uint64_t nd, const uint8_t *__restrict__ cls, unsigned long long *__restrict__ totals)
{
  __shared__ unsigned int h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    h[i] = 0;
  __syncthreads();
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nd; j += (uint64_t)gridDim.x * blockDim.x)
    atomicAdd(&h[cls[j]], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i])
      atomicAdd(&totals[i], (unsigned long long)h[i]);
}

unsigned gridOf(const wb_ctx *c, uint64_t n, int per = 16)
{
  return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + kBlock - 1) / kBlock, (uint64_t)c->sm_count * per));
}

/* ---- host side of the writer ---- */

/* pairwisesum (manysum.cpp:120-154): aligned power-of-two blocks summed as
 * balanced trees, the block totals added from the smallest block up. */
double pairwiseTree(const double *a, size_t n)
{
  return n == 1 ? a[0] : pairwiseTree(a, n / 2) + pairwiseTree(a + n / 2, n / 2);
}

double pairwiseSum(const std::vector<double> &a)
{
  const size_t n = a.size();
  std::vector<double> blocks;   // by bit, low to high
  size_t start = n;
  double sum = 0;
  for (int bit = 0; bit < 64 && (n >> bit); bit++)
    if ((n >> bit) & 1)
    {
      start -= (size_t)1 << bit;
      sum += pairwiseTree(a.data() + start, (size_t)1 << bit);
    }
  return sum;
}

/* manygcd (manygcd.cpp:28-74): the three bubble passes, then subtract the
 * second largest from the largest (or drop the largest when they agree within
 * toler) until all agree; the mean of what is left.  The subtraction makes no
 * progress when a zero (or a value far below the others) sits beside a larger
 * value, and the reference then never returns; here the walk gives up after
 * 2^26 steps and the caller reports it. */
bool manyGcd(std::vector<double> v, double toler, double &out)
{
  for (double &x : v)
    x = std::fabs(x);
  auto up = [&] {
    for (size_t i = 0; i + 1 < v.size(); i++)
      if (v[i] > v[i + 1])
        std::swap(v[i], v[i + 1]);
  };
  auto down = [&] {
    for (long i = (long)v.size() - 2; i >= 0; i--)
      if (v[i] > v[i + 1])
        std::swap(v[i], v[i + 1]);
  };
  out = 0;
  if (v.empty())
    return true;
  up();
  down();
  up();
  long steps = 0;
  while (v.size() && v.back() > v[0] + toler)
  {
    if (++steps > (1l << 26))
      return false;
    const size_t sz = v.size();
    if (v[sz - 1] - v[sz - 2] > toler)
    {
      v[sz - 1] -= v[sz - 2];
      down();
    }
    else
      v.resize(sz - 1);
    up();
  }
  out = v.size() ? pairwiseSum(v) / v.size() : 0;
  return true;
}

/* combine1Scale (las.cpp:906-923). */
bool combineOne(const std::vector<double> &scales, const std::vector<double> &offsets, double &ret)
{
  double toler = INFINITY, sg, og;
  ret = 0;
  for (double s : scales)
    if (std::fabs(s) < toler)
      toler = std::fabs(s);
  toler /= 1e6;
  if (!manyGcd(scales, toler, sg) || !manyGcd(offsets, toler, og))
    return false;
  if ((og > 10.5 * sg || og == 0) && std::fabs(og / sg - std::rint(og / sg)) < 1e-6)
    ret = sg;
  for (int i = 10; i > 0; i--)
    for (int j = 10; j > 0; j--)
      if (std::fabs(sg * i - og * j) < toler)
        ret = sg / j;
  return true;
}

/* LasHeader::setScale (las.cpp:636-673) on one axis. */
void setScale(double lo, double hi, double scale, double unit, double &sc, double &off)
{
  const double minScale = (hi - lo) / 4132485216.;
  off = (lo + hi) / 2 / unit;
  if (scale > minScale && std::isfinite(scale))
  {
    sc = scale / unit;
    off = std::rint(off / sc) * sc;
  }
  else
    sc = minScale / unit;
}

/* CloudOutput::className (cloudoutput.cpp:41-116). */
std::string className(int n)
{
  static const char *names[23] = {"raw",      "nonground", "ground",    "lowveg",    "medveg",  "highveg",
                                  "building", "lownoise",  nullptr,     "water",     "rail",    "road",
                                  "overlap",  "wireguard", "conductor", "tower",     "insulator", "bridge",
                                  "highnoise", "overhead", "ignground", "snow",      "temporal"};
  if (n >= 0 && n < 23 && names[n])
    return names[n];
  return "reserved" + std::to_string(n);
}

/* The sets of files openFiles opens (cloudoutput.cpp:116-185): one set per
 * class of the class totals (class 0 always among them: threads.cpp:430-431)
 * or one set of all points; ceil(total / points_per_file) files per set
 * (one without a limit). */
struct Plan
{
  std::vector<int> setClass;        /* class of each set */
  std::vector<int> setFile0;        /* first file of each set */
  std::vector<int> setFiles;        /* files of each set */
  uint16_t setOf[256];
  int digits = 0;
  int nFiles = 0;
};

Plan planFiles(const uint64_t *tot, const wb_las_output *o)
{
  Plan P;
  uint64_t grand = 0;
  for (int c = 0; c < 256; c++)
    grand += tot[c];
  const uint64_t ppf = o->points_per_file;
  if (ppf)
  {
    uint64_t quot = (grand + ppf - 1) / ppf;
    if (quot)
      quot--;
    if (!quot)
      quot++;
    while (quot)
    {
      quot /= 10;
      P.digits++;
    }
  }
  for (int c = 0; c < 256; c++)
    P.setOf[c] = 0;
  auto addSet = [&](int cls, uint64_t total) {
    const uint64_t quot = ppf ? (total + ppf - 1) / ppf : 1;
    P.setClass.push_back(cls);
    P.setFile0.push_back(P.nFiles);
    P.setFiles.push_back((int)quot);
    P.nFiles += (int)quot;
  };
  if (o->separate_classes)
  {
    for (int c = 0; c < 256; c++)
      if (c == 0 || tot[c])
      {
        P.setOf[c] = (uint16_t)P.setClass.size();
        addSet(c, tot[c]);
      }
  }
  else
    addSet(0, grand);
  return P;
}

bool validOutput(const wb_las_output *o)
{
  if (!o || o->point_format < 0 || o->point_format > 10 || !(o->unit > 0) || !std::isfinite(o->unit))
    return false;
  for (int k = 0; k < 3; k++)
    if (!std::isfinite(o->min_cor[k]) || !std::isfinite(o->max_cor[k]) || !(o->max_cor[k] >= o->min_cor[k]))
      return false;
  return true;
}

void put16(uint8_t *h, int o, uint32_t v)
{
  h[o] = (uint8_t)v;
  h[o + 1] = (uint8_t)(v >> 8);
}
void put32(uint8_t *h, int o, uint32_t v)
{
  put16(h, o, v);
  put16(h, o + 2, v >> 16);
}
void put64(uint8_t *h, int o, uint64_t v)
{
  put32(h, o, (uint32_t)v);
  put32(h, o + 4, (uint32_t)(v >> 32));
}
void putDouble(uint8_t *h, int o, double v)
{
  uint64_t u;
  memcpy(&u, &v, 8);
  put64(h, o, u);
}
}  // namespace

extern "C" {

int wb_las_point_length(int f)
{
  return f >= 0 && f <= 10 ? layoutOf(f).len : 0;
}

int wb_las_join_point_format(const int *formats, int n)
{
  static const int features[11] = {0x0, 0x1, 0x2, 0x3, 0x9, 0xb, 0x101, 0x103, 0x107, 0x109, 0x10f};   // las.cpp:39
  int all = 0;
  for (int i = 0; i < n; i++)
    if (formats && formats[i] >= 0 && formats[i] < 11)
      all |= features[formats[i]];
  for (int i = 0; i < 11; i++)
    if ((all | features[i]) == features[i])
      return i;
  return WB_EINVAL;
}

int wb_las_combine_scales(const double *scales, const double *offsets, int n, double *out)
{
  if (!scales || !offsets || !out || n <= 0)
    return WB_EINVAL;
  for (int k = 0; k < 3; k++)
  {
    std::vector<double> s(n), o(n);
    for (int i = 0; i < n; i++)
    {
      s[i] = scales[i * 3 + k];
      o[i] = offsets[i * 3 + k];
    }
    if (!combineOne(s, o, out[k]))
      return WB_EINVAL;   // the reference's manygcd would not return
  }
  return 0;
}

int wb_las_decode(wb_ctx *c, const wb_cloud *cloud, int fmt, const wb_las_points *out)
{
  if (!c || !cloud || !out || (cloud->n && !cloud->records))
    return WB_EINVAL;
  if (fmt < 0 || fmt > 10 || cloud->stride < (uint32_t)layoutOf(fmt).len)
    return wb_fail(c, WB_EINVAL, "wb_las_decode: point format 0-10 and a stride that holds its record");
  const uint64_t n = cloud->n;
  if (!n)
    return 0;
  if (cloud->device_resident && !wb_device_accessible(cloud->records))
    return wb_fail(c, WB_EINVAL, "wb_las_decode: device_resident records must be device memory");
  WbDeviceGuard deviceGuard(c->device);
  int rc;
  DecodeArgs a;
  a.n = n;
  a.stride = cloud->stride;
  a.fmt = fmt;
  for (int k = 0; k < 3; k++)
  {
    a.d.off[k] = cloud->offset[k];
    a.d.scale[k] = cloud->scale[k];
  }
  a.d.unit = cloud->unit;
  WbScratch rin(c), fields(c);
  const bool host = !cloud->device_resident;
  a.rec = (const uint8_t *)cloud->records;
  a.o = *out;
  // with host records and arrays: the records go up, the wanted fields come
  // back from device arrays carved out of one buffer
  struct Field
  {
    void *host;
    void **dev;
    size_t size;
  };
  wb_las_points &o = a.o;
  Field fs[] = {{out->x, (void **)&o.x, 8},
                {out->y, (void **)&o.y, 8},
                {out->z, (void **)&o.z, 8},
                {out->intensity, (void **)&o.intensity, 2},
                {out->return_num, (void **)&o.return_num, 2},
                {out->n_returns, (void **)&o.n_returns, 2},
                {out->scan_direction, (void **)&o.scan_direction, 1},
                {out->edge_line, (void **)&o.edge_line, 1},
                {out->classification, (void **)&o.classification, 2},
                {out->class_flags, (void **)&o.class_flags, 2},
                {out->scanner_channel, (void **)&o.scanner_channel, 2},
                {out->user_data, (void **)&o.user_data, 2},
                {out->scan_angle, (void **)&o.scan_angle, 4},
                {out->point_source, (void **)&o.point_source, 2},
                {out->gps_time, (void **)&o.gps_time, 8},
                {out->red, (void **)&o.red, 2},
                {out->green, (void **)&o.green, 2},
                {out->blue, (void **)&o.blue, 2},
                {out->nir, (void **)&o.nir, 2}};
  if (host)
  {
    if ((rc = wb_ensure(c, rin.b, n * cloud->stride)))
      return rc;
    WB_CUDA(c, cudaMemcpyAsync(rin.b.p, cloud->records, n * cloud->stride, cudaMemcpyDefault, c->stream));
    a.rec = (const uint8_t *)rin.b.p;
    size_t total = 0;
    for (Field &f : fs)
      if (f.host)
        total += (n * f.size + 255) & ~(size_t)255;
    if (total && (rc = wb_ensure(c, fields.b, total)))
      return rc;
    size_t at = 0;
    for (Field &f : fs)
      if (f.host)
      {
        *f.dev = (uint8_t *)fields.b.p + at;
        at += (n * f.size + 255) & ~(size_t)255;
      }
  }
  if ((rc = angleTables(c, a.t)))
    return rc;
  a.words = ((uintptr_t)a.rec % 4 == 0) && (a.stride % 4 == 0);
  a.vec16 = (uintptr_t)a.rec % 16 == 0;
  { decodeKernel<<<gridOf(c, n), kBlock, 0, c->stream>>>(a); ++c->launches; }
  cudaError_t e = cudaGetLastError();
  if (host)
    for (Field &f : fs)
      if (f.host && e == cudaSuccess)
        e = cudaMemcpyAsync(f.host, *f.dev, n * f.size, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess)
    return wb_fail(c, WB_ECUDA, std::string("wb_las_decode: ") + cudaGetErrorString(e));
  return 0;
}

int wb_las_write_output(wb_ctx *c, const wb_cloud *cloud, int in_format, const uint8_t *cls,
                        const wb_las_output *opt, void *out, int out_on_device, wb_las_file *files, int max_files,
                        int *n_files)
{
  if (!c || !cloud || !n_files || (cloud->n && !cloud->records))
    return WB_EINVAL;
  *n_files = 0;
  if (!validOutput(opt))
    return wb_fail(c, WB_EINVAL, "wb_las_write_output: output format 0-10, a positive unit and finite corners");
  if (in_format < 0 || in_format > 10 || cloud->stride < (uint32_t)layoutOf(in_format).len)
    return wb_fail(c, WB_EINVAL, "wb_las_write_output: input format 0-10 and a stride that holds its record");
  if (c->stage < 1 || cloud->n != c->n)
    return wb_fail(c, WB_ESTATE, "wb_las_write_output: build the octree of this cloud first");
  if (!cls && (c->stage < 3 || !c->clsFinal))
    return wb_fail(c, WB_ESTATE, "wb_las_write_output: no class bytes (classify first or pass them)");
  if (c->nd && !out)
    return wb_fail(c, WB_EINVAL, "wb_las_write_output: no output buffer");
  if (c->nd && out_on_device && !wb_device_accessible(out))
    return wb_fail(c, WB_EINVAL, "wb_las_write_output: out_on_device needs a device pointer");
  if (cloud->device_resident && c->n &&
      (!wb_device_accessible(cloud->records) || (cls && !wb_device_accessible(cls))))
    return wb_fail(c, WB_EINVAL, "wb_las_write_output: device_resident records (and class bytes) must be device memory");
  WbDeviceGuard deviceGuard(c->device);
  const uint64_t n = c->n, nd = c->nd, L = c->n_leaves;
  const Layout Li = layoutOf(in_format), Lo = layoutOf(opt->point_format);
  int rc;
  WbScratch rin(c), cin(c), cstore(c), dout(c), tot(c), counts(c), bases(c), fileOf(c), stats(c);

  WriteArgs a;
  a.stride = cloud->stride;
  a.inFmt = in_format;
  a.outFmt = opt->point_format;
  for (int k = 0; k < 3; k++)
  {
    a.d.off[k] = cloud->offset[k];
    a.d.scale[k] = cloud->scale[k];
  }
  a.d.unit = cloud->unit;
  // one scale and offset for every file: setScale gets the same box each time
  for (int k = 0; k < 3; k++)
    setScale(opt->min_cor[k], opt->max_cor[k], opt->scale[k], opt->unit, a.e.scale[k], a.e.off[k]);
  a.e.unit = opt->unit;
  for (int k = 0; k < 3; k++)
  {
    a.e.inv[k] = 1 / a.e.scale[k];
    // Same unit and scale in and out: writePoint's integer is X + D whenever
    // delta = (offset_in - offset_out)/scale lies within 1/4 - err of the
    // integer D, err bounding every rounding of decode and re-encode over the
    // whole int32 range (a few units of 2^-53 times the magnitudes involved).
    a.e.shift[k] = false;
    a.e.by[k] = 0;
    if (cloud->unit == opt->unit && cloud->scale[k] == a.e.scale[k] && a.e.scale[k] > 0)
    {
      const double delta = (cloud->offset[k] - a.e.off[k]) / a.e.scale[k];
      const double D = std::rint(delta);
      const double err = 8 * 0x1p-53 *
                         (4294967296.0 + (std::fabs(cloud->offset[k]) + std::fabs(a.e.off[k])) / a.e.scale[k] +
                          std::fabs(delta));
      if (std::isfinite(delta) && std::fabs(D) < 0x1p60 && std::fabs(delta - D) + err < 0.25)
      {
        a.e.shift[k] = true;
        a.e.by[k] = (long long)D;
      }
    }
  }
  if ((rc = angleTables(c, a.t)))
    return rc;
  for (int k = 0; k < 3; k++)
    if (!(a.e.scale[k] > 0) || !std::isfinite(a.e.scale[k]))
      return wb_fail(c, WB_EINVAL, "wb_las_write_output: the output box and scale give no positive record scale");

  if (cloud->device_resident)
    a.rec = (const uint8_t *)cloud->records;
  else if (n)
  {
    if ((rc = wb_ensure(c, rin.b, n * cloud->stride)))
      return rc;
    WB_CUDA(c, cudaMemcpyAsync(rin.b.p, cloud->records, n * cloud->stride, cudaMemcpyDefault, c->stream));
    a.rec = (const uint8_t *)rin.b.p;
  }
  else
    a.rec = nullptr;
  a.inWords = ((uintptr_t)a.rec % 4 == 0) && (a.stride % 4 == 0);
  const uint8_t *recCls;
  if (!cls)
    recCls = c->clsFinal;
  else if (cloud->device_resident)
    recCls = cls;
  else
  {
    if ((rc = wb_ensure(c, cin.b, n + 16)))
      return rc;
    WB_CUDA(c, cudaMemcpyAsync(cin.b.p, cls, n, cudaMemcpyDefault, c->stream));
    recCls = (const uint8_t *)cin.b.p;
  }
  a.sidx = (const uint32_t *)c->sidx.p;
  // class bytes in store order, read sequentially by every pass below
  if ((rc = wb_ensure(c, cstore.b, nd + 16)))
    return rc;
  if (nd)
    { storeClassKernel<<<gridOf(c, nd), kBlock, 0, c->stream>>>(
          nd, a.sidx, (!cls && c->stage >= 3) ? (const int32_t *)c->owner.p : nullptr, (const uint8_t *)c->label.p, recCls,
          (uint8_t *)cstore.b.p); ++c->launches; }
  a.cls = (const uint8_t *)cstore.b.p;
  a.leafFirst = (const uint32_t *)c->leafFirst.p;
  a.leafCount = (const uint32_t *)c->leafCount.p;
  a.nLeaves = L;

  // class totals of the stored points (OctStore::countClasses)
  if ((rc = wb_ensure(c, tot.b, 256 * 8)))
    return rc;
  WB_CUDA(c, cudaMemsetAsync(tot.b.p, 0, 256 * 8, c->stream));
  if (nd)
    { storedTotals<<<gridOf(c, nd), kBlock, 0, c->stream>>>(nd, a.cls, (unsigned long long *)tot.b.p); ++c->launches; }
  uint64_t T[256];
  WB_CUDA(c, cudaMemcpyAsync(T, tot.b.p, sizeof T, cudaMemcpyDefault, c->stream));
  WB_CUDA(c, cudaStreamSynchronize(c->stream));

  Plan P = planFiles(T, opt);
  *n_files = P.nFiles;
  if (!files || max_files < P.nFiles)
    return wb_fail(c, WB_EINVAL, "wb_las_write_output: room for " + std::to_string(P.nFiles) + " files needed");
  const uint32_t S = (uint32_t)P.setClass.size();
  a.nSets = S;
  memcpy(a.setOf, P.setOf, sizeof a.setOf);
  a.nFiles = (uint32_t)P.nFiles;

  // stored points per (block, set)
  // per (block, set) counts, first records and files go through one pinned
  // host buffer of the context (16 bytes per entry)
  const size_t stageBytes = L * S * 16 + 64;
  if (c->hostStageCap < stageBytes)
  {
    WB_CUDA(c, cudaStreamSynchronize(c->stream));
    if (c->hostStage)
      cudaFreeHost(c->hostStage);
    c->hostStage = nullptr;
    c->hostStageCap = 0;
    WB_CUDA(c, cudaHostAlloc(&c->hostStage, stageBytes, cudaHostAllocDefault));
    c->hostStageCap = stageBytes;
  }
  uint64_t *base = (uint64_t *)c->hostStage;
  uint32_t *cnt = (uint32_t *)(base + L * S), *fof = cnt + L * S;
  if (L)
  {
    if ((rc = wb_ensure(c, counts.b, L * S * 4)))
      return rc;
    WB_CUDA(c, cudaMemsetAsync(counts.b.p, 0, L * S * 4, c->stream));
    { setCountKernel<<<gridOf(c, L * 32, 8), kBlock, 0, c->stream>>>(a, (uint32_t *)counts.b.p); ++c->launches; }
    WB_CUDA(c, cudaMemcpyAsync(cnt, counts.b.p, L * S * 4, cudaMemcpyDefault, c->stream));
    WB_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  memset(base, 0, L * S * 8);
  memset(fof, 0, L * S * 4);

  // writeFiles: at each block, each set's points go to its file holding the
  // fewest points, the first of them on a tie (cloudoutput.cpp:196-209)
  std::vector<uint64_t> fileCount(P.nFiles, 0);
  typedef std::pair<uint64_t, int> Entry;
  for (uint32_t s = 0; s < S; s++)
  {
    const int f0 = P.setFile0[s], nf = P.setFiles[s];
    std::priority_queue<Entry, std::vector<Entry>, std::greater<Entry>> heap;
    if (nf > 16)
      for (int i = 0; i < nf; i++)
        heap.push(Entry(0, f0 + i));
    for (uint64_t leaf = 0; leaf < L; leaf++)
    {
      const uint32_t k = cnt[leaf * S + s];
      if (!k)
        continue;
      if (!nf)
        return wb_fail(c, WB_ESTATE, "wb_las_write_output: points of a class without a file");
      int f = f0;
      if (nf > 16)
      {
        f = heap.top().second;
        heap.pop();
      }
      else
        for (int i = 1; i < nf; i++)
          if (fileCount[f0 + i] < fileCount[f])
            f = f0 + i;
      base[leaf * S + s] = fileCount[f];
      fof[leaf * S + s] = (uint32_t)f;
      fileCount[f] += k;
      if (nf > 16)
        heap.push(Entry(fileCount[f], f));
    }
  }
  std::vector<uint64_t> fileFirst(P.nFiles + 1, 0);
  for (int f = 0; f < P.nFiles; f++)
    fileFirst[f + 1] = fileFirst[f] + fileCount[f];
  for (uint64_t i = 0; i < L * S; i++)
    base[i] += fileFirst[fof[i]];

  uint8_t *dst = (uint8_t *)out;
  const uint64_t outBytes = nd * (uint64_t)Lo.len;
  if (!out_on_device && outBytes)
  {
    if ((rc = wb_ensure(c, dout.b, outBytes)))
      return rc;
    dst = (uint8_t *)dout.b.p;
  }
  a.out = dst;
  a.outWidth = ((uintptr_t)dst % 4 == 0 && Lo.len % 4 == 0) ? 4 : (((uintptr_t)dst % 2 == 0 && Lo.len % 2 == 0) ? 2 : 1);
  if ((rc = wb_ensure(c, stats.b, sizeof(FileStat) * (P.nFiles + 1))))
    return rc;
  a.stats = (FileStat *)stats.b.p;
  { statInit<<<gridOf(c, P.nFiles + 1), kBlock, 0, c->stream>>>(a.stats, (uint32_t)P.nFiles); ++c->launches; }
  if (L && nd)
  {
    if ((rc = wb_ensure(c, bases.b, L * S * 8)) || (rc = wb_ensure(c, fileOf.b, L * S * 4)))
      return rc;
    WB_CUDA(c, cudaMemcpyAsync(bases.b.p, base, L * S * 8, cudaMemcpyDefault, c->stream));
    WB_CUDA(c, cudaMemcpyAsync(fileOf.b.p, fof, L * S * 4, cudaMemcpyDefault, c->stream));
    a.base = (unsigned long long *)bases.b.p;
    a.fileOf = (const uint32_t *)fileOf.b.p;
    const size_t slots = 2 * (size_t)kBlock * kSlotWords * 4;
    if (P.nFiles <= kSharedFiles)
    {
      const size_t smem = slots + sizeof(FileStat) * kSharedFiles;
      WB_CUDA(c, cudaFuncSetAttribute(writeKernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      { writeKernel<true><<<gridOf(c, L * 32, 4), kBlock, smem, c->stream>>>(a); ++c->launches; }
    }
    else
    {
      WB_CUDA(c, cudaFuncSetAttribute(writeKernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)slots));
      { writeKernel<false><<<gridOf(c, L * 32, 4), kBlock, slots, c->stream>>>(a); ++c->launches; }
    }
  }
  std::vector<FileStat> fs(P.nFiles + 1);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(fs.data(), a.stats, sizeof(FileStat) * (P.nFiles + 1), cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess && !out_on_device && outBytes)
    e = cudaMemcpyAsync(out, dst, outBytes, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess)
    return wb_fail(c, WB_ECUDA, std::string("wb_las_write_output: ") + cudaGetErrorString(e));

  for (uint32_t s = 0; s < S; s++)
    for (int i = 0; i < P.setFiles[s]; i++)
    {
      const int f = P.setFile0[s] + i;
      wb_las_file &F = files[f];
      memset(&F, 0, sizeof F);
      F.class_id = P.setClass[s];
      F.index = i;
      F.name_digits = P.digits;
      F.point_format = opt->point_format;
      F.first = fileFirst[f];
      for (int k = 0; k < 16; k++)
        F.n_points[k] = fs[f].cnt[k];
      for (int k = 0; k < 3; k++)
      {
        F.scale[k] = a.e.scale[k];
        F.offset[k] = a.e.off[k];
        // writtenX = xInt*xScale + xOffset (las.cpp:830-845), monotone in xInt
        F.min[k] = F.n_points[0] ? (double)fs[f].mn[k] * a.e.scale[k] + a.e.off[k] : INFINITY;
        F.max[k] = F.n_points[0] ? (double)fs[f].mx[k] * a.e.scale[k] + a.e.off[k] : -INFINITY;
      }
      if (F.n_points[0] != fileCount[f])
        return wb_fail(c, WB_ESTATE, "wb_las_write_output: file counts disagree");
    }
  return 0;
}

int wb_las_header_bytes(const wb_las_output *opt, const wb_las_file *f, uint8_t *h)
{
  if (!opt || !f || !h || f->point_format < 0 || f->point_format > 10)
    return WB_EINVAL;
  memset(h, 0, 375);
  h[0] = 'L';
  h[1] = 'A';
  h[2] = 'S';
  h[3] = 'F';
  h[24] = 1;   // version 1.4 (CloudOutput::openFiles sets it)
  h[25] = 4;
  const char *sys = opt->separate_classes ? "EXTRACTION" : (opt->n_input_files > 1 ? "MERGE" : "MODIFICATION");
  strncpy((char *)h + 26, sys, 32);
  const char *sw = opt->software ? opt->software : "Wolkenbase 0.1.2~alpha";
  strncpy((char *)h + 58, sw, 32);
  int day = opt->creation_day, year = opt->creation_year;
  if (!year)
  {
    time_t now = time(nullptr);
    struct tm t;
    gmtime_r(&now, &t);
    day = t.tm_yday + 1;
    year = t.tm_year + 1900;
  }
  put16(h, 90, (uint32_t)day);
  put16(h, 92, (uint32_t)year);
  put16(h, 94, 375);   // headerSize and pointOffset (setVersion, las.cpp:613-625)
  put32(h, 96, 375);
  put32(h, 100, 0);
  h[104] = (uint8_t)f->point_format;
  const int len = layoutOf(f->point_format).len;
  put16(h, 105, (uint32_t)len);
  bool legacy = true;   // writeHeader, las.cpp:542-551
  for (int i = 0; i < 6; i++)
    if (f->n_points[i] > 4294967295ull)
      legacy = false;
  for (int i = 6; i < 16; i++)
    if (f->n_points[i] > 0)
      legacy = false;
  for (int i = 0; i < 6; i++)
    put32(h, 107 + 4 * i, legacy ? (uint32_t)f->n_points[i] : 0);
  for (int k = 0; k < 3; k++)
  {
    putDouble(h, 131 + 8 * k, f->scale[k]);
    putDouble(h, 155 + 8 * k, f->offset[k]);
    putDouble(h, 179 + 16 * k, f->max[k]);
    putDouble(h, 187 + 16 * k, f->min[k]);
  }
  put64(h, 227, 0);
  // start of the extended variable length records: the end of the points
  put64(h, 235, f->n_points[0] ? 375 + f->n_points[0] * (uint64_t)len : 0);
  put32(h, 243, 0);
  for (int i = 0; i < 16; i++)
    put64(h, 247 + 8 * i, f->n_points[i]);
  return 0;
}

int wb_las_file_name(const wb_las_output *opt, const wb_las_file *f, const char *base, char *buf, size_t cap)
{
  if (!opt || !f || !base || !buf || !cap)
    return WB_EINVAL;
  std::string name = base;
  if (opt->separate_classes)
    name += "-" + className(f->class_id);
  if (opt->points_per_file)
    name += "-";
  if (f->name_digits)
  {
    char num[32];
    snprintf(num, sizeof num, "%0*d", f->name_digits, f->index);
    name += num;
  }
  name += ".las";
  if (name.size() + 1 > cap)
    return WB_EINVAL;
  memcpy(buf, name.c_str(), name.size() + 1);
  return 0;
}

int wb_las_write_files(wb_ctx *c, const wb_cloud *cloud, int in_format, const uint8_t *cls, const wb_las_output *opt,
                       const char *base, wb_las_file *files, int max_files, int *n_files)
{
  if (!c || !cloud || !opt || !base || !n_files)
    return WB_EINVAL;
  if (!validOutput(opt))
    return wb_fail(c, WB_EINVAL, "wb_las_write_files: output format 0-10, a positive unit and finite corners");
  const size_t len = (size_t)layoutOf(opt->point_format).len;
  std::vector<uint8_t> recs(c->nd * len);
  int rc = wb_las_write_output(c, cloud, in_format, cls, opt, recs.data(), 0, files, max_files, n_files);
  if (rc)
    return rc;
  for (int f = 0; f < *n_files; f++)
  {
    char name[4096];
    uint8_t hdr[375];
    if (wb_las_file_name(opt, &files[f], base, name, sizeof name) || wb_las_header_bytes(opt, &files[f], hdr))
      return wb_fail(c, WB_EINVAL, "wb_las_write_files: file name too long");
    FILE *fp = fopen(name, "wb");
    if (!fp)
      return wb_fail(c, WB_EIO, std::string("wb_las_write_files: cannot open ") + name);
    const size_t bytes = files[f].n_points[0] * len;
    bool ok = fwrite(hdr, 1, 375, fp) == 375 &&
              (!bytes || fwrite(recs.data() + files[f].first * len, 1, bytes, fp) == bytes);
    ok = (fclose(fp) == 0) && ok;
    if (!ok)
      return wb_fail(c, WB_EIO, std::string("wb_las_write_files: cannot write ") + name);
  }
  return 0;
}

}  // extern "C"

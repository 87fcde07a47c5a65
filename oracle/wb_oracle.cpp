/* CPU restatement of wolkenbase's hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm as
 * the checker.  The product library never links or calls it.  Each section
 * cites the reference function it restates (paths relative to the
 * phma/wolkenbase source tree).  The restatement is pinned against the
 * reference's own sources compiled here (oracle/_ref/wb_ref) by
 * tests/test_oracle_golden.py.
 *
 * Deliberate differences from the reference, none of which changes a result:
 *  - classifyCylinder visits downPoints in index order instead of the
 *    relprime stride (classify.cpp:140-156); the stride only changes how soon
 *    the early exit fires, and the surround test is monotone in the set.
 *  - surround() uses pruning parity 0 instead of time(nullptr)&1
 *    (classify.cpp:73); pruning only removes middles of <30 degree triples,
 *    which can never open a 144 degree gap.
 *  - Scan and classify run tiles on several threads; the "last tile in
 *    flowsnake order wins" rule of the serial driver is kept by resolving
 *    each point's class with the largest flowsnake counter that classified it.
 */
#include "wb_oracle.h"
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

const int kRecords = 537;                        // octree.h:40-42 (no WAVEFORM)
const int kDeg30 = 0x0aaaaaab, kDeg45 = 0x10000000, kDeg90 = 0x20000000;
const int kDeg144 = 0x33333333, kDeg180 = 0x40000000, kDeg270 = 0x60000000;
const double kSqrt34 = 0.86602540378443864676372317;   // sqrt(3)/2
const double kSqrt7 = 2.6457513110645905905016;

double nowSec()
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

inline double sq(double x) { return x * x; }
inline double cube3(double x) { return x * x * x; }

/* The C library hypot that the reference calls (point.cpp:189-192,
 * shape.cpp:127-135, 214-218) is, in the x86-64 glibc the oracle is pinned
 * against, the corrected square root of Borges, "An Improved Algorithm for
 * hypot(a,b)" (2019), non-fused form.  Restating it here keeps the oracle's
 * results identical on hosts whose libm uses the fused form instead. */
double hypotR(double a, double b)
{
  double ax = fabs(a), ay = fabs(b);
  if (ay > ax)
    std::swap(ax, ay);
  if (ay == 0)
    return ax;
  double h = sqrt(ax * ax + ay * ay), t1, t2;
  if (h <= 2.0 * ay)
  {
    double d = h - ay;
    t1 = ax * (2.0 * d - ax);
    t2 = (d - 2.0 * (ax - ay)) * d;
  }
  else
  {
    double d = h - ax;
    t1 = 2.0 * d * (ax - 2.0 * ay);
    t2 = (4.0 * d - ay) * ay + d * d;
  }
  return h - (t1 + t2) / (2.0 * h);
}

/* ---------------- integer angles (angle.cpp:117-155, 305-320) ---------------- */

double gTan[511], gSin[512], gCos[512];
bool gTablesSet = false;

long double angleRad(int angle) { return (long double)angle * M_PIl / 1073741824.; }
double sinInt(int angle) { return (double)sinl(angleRad(angle)); }
double cosInt(int angle) { return (double)cosl(angleRad(angle)); }
double tanInt(int angle) { return (double)tanl(angleRad(angle)); }

void fillTables()
{
  for (int i = 0; i < 511; i++)
    gTan[i] = tanInt(i * 0x100000 - 0xff00000);
  for (int i = 0; i < 512; i++)
  {
    gSin[i] = sinInt(i * 0x100000 - 0xff80000);
    gCos[i] = cosInt(i * 0x100000 - 0xff80000);
  }
  gTablesSet = true;
}

void ensureTables()
{
  if (!gTablesSet)
    fillTables();
}

int atan2iR(double y, double x)
{
  int ret = 0, h;
  double t;
  if (x < 0)
  {
    ret += (y > 0) ? kDeg180 : -kDeg180;
    y = -y;
    x = -x;
  }
  if (y > x)
  {
    ret += kDeg90;
    std::swap(x, y);
    y = -y;
  }
  if (-y > x)
  {
    ret -= kDeg90;
    std::swap(x, y);
    x = -x;
  }
  t = y / x;
  for (h = kDeg45 / 2; h > kDeg45 / 1024; h /= 2)
    if (t > gTan[(((ret + kDeg45) & 0x1ff00000) >> 20) - 1])
      ret += h;
    else
      ret -= h;
  h = 511 - (((ret + kDeg45) & 0x1ff00000) >> 20);
  t = x * gCos[h] - y * gSin[h];
  y = y * gCos[h] + x * gSin[h];
  x = t;
  long double corr = 0x40000000 / M_PIl * y / x - 1.1392738508503886e8 * cube3(y / x);
  ret += (int)lrintl(corr);
  if (x == 0 && y == 0)
    ret = 0;
  return ret;
}

/* ---------------- pairwise sum and 3-column least squares ----------------
 * manysum.cpp:120-154 (pairwisesum), matrix.cpp:181-215 (transmult, *),
 * matrix.cpp:262-422 (rowop, gausselim, findpivot), leastsquares.cpp:28-43. */

double pairwise(const double *a, unsigned n)
{
  double part[32], total = 0;
  unsigned i = 0;
  // Groups of eight are added as a fixed tree; completed power-of-two runs
  // are merged like a binary counter.
  for (; i + 7 < n; i += 8)
  {
    double g = (((a[i] + a[i + 1]) + (a[i + 2] + a[i + 3])) + ((a[i + 4] + a[i + 5]) + (a[i + 6] + a[i + 7])));
    unsigned carry = i ^ (i + 8);
    if (carry == 8)
      part[3] = g;
    else
    {
      part[3] += g;
      unsigned lvl = 4;
      for (; carry >> (lvl + 1); lvl++)
        part[lvl] += part[lvl - 1];
      part[lvl] = part[lvl - 1];
    }
  }
  for (; i < n; i++)
  {
    unsigned carry = i ^ (i + 1);
    if (carry == 1)
      part[0] = a[i];
    else
    {
      part[0] += a[i];
      unsigned lvl = 1;
      for (; carry >> (lvl + 1); lvl++)
        part[lvl] += part[lvl - 1];
      part[lvl] = part[lvl - 1];
    }
  }
  for (i = 0; i < 32; i++)
    if ((n >> i) & 1)
      total += part[i];
  return total;
}

struct Mat3
{
  double m[3][3];
  double b[3];
};

void swapRows(Mat3 &s, int r0, int r1)
{
  for (int k = 0; k < 3; k++)
    std::swap(s.m[r0][k], s.m[r1][k]);
  std::swap(s.b[r0], s.b[r1]);
}

void findPivot(Mat3 &s, int row, int column)
{
  int pivotrow = -1;
  double maxratio = 0;
  for (; pivotrow < row && column < 3; column++)
  {
    for (int i = row; i < 3; i++)
    {
      double sqs[3] = {0, 0, 0};
      for (int j = column + 1; j < 3; j++)
        sqs[j - column - 1] = sq(s.m[i][j]);
      double ratio = sq(s.m[i][column]) / pairwise(sqs, 3 - column);
      if (ratio > maxratio)
      {
        pivotrow = i;
        maxratio = ratio;
      }
    }
  }
  if (pivotrow > row)
    swapRows(s, pivotrow, row);
}

void rowOp(Mat3 &s, int row0, int row1, int piv)
{
  double *r0 = s.m[row0], *r1 = s.m[row1];
  double slope = 0, minslope = INFINITY, detfactor;
  int flags = 0, pivot;
  if (piv >= 0 && r0[piv] == 0 && r1[piv] == 0)
    piv = -1;
  pivot = piv;
  if (piv >= 0 && r0[piv] == 0)
    flags = 9;
  for (int i = 0; piv < 0 && i < 3; i++)
    if (r0[i] != 0 || r1[i] != 0)
    {
      if (fabs(r0[i]) > fabs(r1[i]) || row0 >= row1)
      {
        slope = fabs(r1[i] / r0[i]);
        flags &= ~8;
      }
      else
      {
        slope = fabs(r0[i] / r1[i]);
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
    swapRows(s, row0, row1);
  detfactor = pivot < 0 ? 0 : r0[pivot];
  if (detfactor != 0 && detfactor != 1)
  {
    for (int i = 0; i < 3; i++)
      r0[i] /= detfactor;
    s.b[row0] /= detfactor;
  }
  if (pivot >= 0)
    slope = r1[pivot];
  if (slope != 0 && row0 != row1)
  {
    for (int i = 0; i < 3; i++)
      r1[i] -= r0[i] * slope;
    s.b[row1] -= s.b[row0] * slope;
  }
}

/* Plane z = a*x + b*y + c through rows (x, y, z); returns (a, b, c). */
void lsqPlane(const double *x, const double *y, const double *z, unsigned n, double out[3])
{
  std::vector<double> t(n);
  const double *cols[3] = {x, y, nullptr};
  Mat3 s;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j <= i; j++)
    {
      for (unsigned k = 0; k < n; k++)
        t[k] = (cols[i] ? cols[i][k] : 1.0) * (cols[j] ? cols[j][k] : 1.0);
      s.m[i][j] = s.m[j][i] = pairwise(t.data(), n);
    }
  for (int i = 0; i < 3; i++)
  {
    for (unsigned k = 0; k < n; k++)
      t[k] = (cols[i] ? cols[i][k] : 1.0) * z[k];
    s.b[i] = pairwise(t.data(), n);
  }
  for (int i = 0; i < 3; i++)
  {
    findPivot(s, i, i);
    for (int j = 0; j < 3; j++)
      rowOp(s, i, j, i);
  }
  for (int i = 2; i >= 0; i--)
    for (int j = 0; j < i; j++)
      rowOp(s, i, j, i);
  for (int i = 0; i < 3; i++)
  {
    out[i] = s.b[i];
    if (s.m[i][i] == 0)
      out[i] = NAN;
  }
}

/* ---------------- shapes (shape.cpp) ---------------- */

struct V3
{
  double x, y, z;
};

struct CubeR
{
  V3 c;
  double side;
  V3 corner(int n) const
  {
    double h = side / 2;
    return V3{(n & 1) ? c.x + h : c.x - h, (n & 2) ? c.y + h : c.y - h, (n & 4) ? c.z + h : c.z - h};
  }
};

double clampToward(double target, double ctr, double side)
{
  if (fabs(target - ctr) < side / 2)
    return target;
  return target > ctr ? ctr + side / 2 : ctr - side / 2;
}

struct Shape
{
  virtual bool in(const V3 &p) const = 0;
  virtual V3 closest(const CubeR &c) const = 0;
  bool inCube(const CubeR &c) const
  {
    bool r = true;
    for (int i = 0; i < 8; i++)
      r = r && in(c.corner(i));
    return r;
  }
  bool meets(const CubeR &c) const { return in(closest(c)); }
  virtual ~Shape() {}
};

struct HyperboloidR : Shape
{
  V3 ctr;
  double por2, slope;
  HyperboloidR(V3 v, double r, double s)
  {
    double por = r * sq(s);
    slope = s;
    por2 = sq(por);
    ctr = V3{v.x + 0, v.y + 0, v.z + por};
  }
  bool in(const V3 &p) const override
  {
    double xyd = hypotR(ctr.x - p.x, ctr.y - p.y);
    double zd = ctr.z - p.z;
    if (slope > 0)
      return zd > 0 && sq(zd) - sq(xyd * slope) >= por2;
    return zd < 0 && sq(zd) - sq(xyd * slope) >= por2;
  }
  V3 closest(const CubeR &c) const override
  {
    V3 r{clampToward(ctr.x, c.c.x, c.side), clampToward(ctr.y, c.c.y, c.side), c.c.z};
    if (slope > 0)
      r.z -= c.side / 2;
    if (slope < 0)
      r.z += c.side / 2;
    return r;
  }
};

struct CylinderR : Shape
{
  double cx, cy, r;
  CylinderR(double x, double y, double rad) : cx(x), cy(y), r(rad) {}
  bool in(const V3 &p) const override { return hypotR(cx - p.x, cy - p.y) <= r; }
  V3 closest(const CubeR &c) const override
  {
    return V3{clampToward(cx, c.c.x, c.side), clampToward(cy, c.c.y, c.side), c.c.z};
  }
};

/* ---------------- octree and block store (octree.cpp) ---------------- */

struct Node
{
  V3 c;
  double side;
  uint64_t sub[8];   // 0 empty, (block<<1)|1 leaf block, node<<1 child node
};

struct Store
{
  std::vector<V3> loc;
  std::vector<Node> nodes;                    // nodes[0] is the root
  std::vector<std::vector<uint32_t>> blocks;  // storage order
  /* the coordinates of blocks[b]'s points in the same order, kept during the
     build so that the de-duplication scan reads one block's memory in
     sequence instead of one random location per stored point */
  std::vector<std::vector<V3>> bloc;
  /* per block, an open-addressing table of positions (+1) in bloc[b] keyed by
     the coordinates: finds the equal point the reference's linear scan finds,
     without reading the whole block */
  static const int kHash = 1024;
  std::vector<std::vector<uint16_t>> bhash;
  std::vector<uint32_t> spill;                // thread buffer 0 (LIFO)

  static uint32_t hashOf(const V3 &p)
  {
    // +0.0 and -0.0 compare equal, so they must hash alike
    double c[3] = {p.x == 0 ? 0.0 : p.x, p.y == 0 ? 0.0 : p.y, p.z == 0 ? 0.0 : p.z};
    uint64_t h = 1469598103934665603ull;
    for (double v : c)
    {
      uint64_t u;
      memcpy(&u, &v, 8);
      h = (h ^ u) * 1099511628211ull;
      h ^= h >> 29;
    }
    return (uint32_t)(h ^ (h >> 32));
  }

  static int octant(const Node &nd, const V3 &p)
  {
    return (p.z >= nd.c.z) * 4 + (p.y >= nd.c.y) * 2 + (p.x >= nd.c.x);
  }
  static CubeR octCube(const Node &nd, int i)
  {
    int xb = i & 1, yb = (i & 2) / 2, zb = (i & 4) / 4;
    return CubeR{V3{nd.c.x + (2 * xb - 1) * nd.side / 4, nd.c.y + (2 * yb - 1) * nd.side / 4,
                    nd.c.z + (2 * zb - 1) * nd.side / 4}, nd.side / 2};
  }
  int64_t findBlock(const V3 &p) const
  {
    size_t k = 0;
    while (true)
    {
      uint64_t s = nodes[k].sub[octant(nodes[k], p)];
      if (s == 0)
        return -1;
      if (s & 1)
        return (int64_t)(s >> 1);
      k = s >> 1;
    }
  }
  CubeR findCube(const V3 &p) const
  {
    size_t k = 0;
    while (true)
    {
      int i = octant(nodes[k], p);
      uint64_t s = nodes[k].sub[i];
      if (s == 0 || (s & 1))
        return octCube(nodes[k], i);
      k = s >> 1;
    }
  }
  void setBlock(const V3 &p, int64_t blk)
  {
    size_t k = 0;
    while (true)
    {
      int i = octant(nodes[k], p);
      uint64_t s = nodes[k].sub[i];
      if (s == 0)
      {
        nodes[k].sub[i] = ((uint64_t)blk << 1) | 1;
        return;
      }
      if (s & 1)
        return;   // occupied; the reference prints an error here
      k = s >> 1;
    }
  }
  void splitAt(const V3 &p)
  {
    size_t k = 0;
    while (true)
    {
      int i = octant(nodes[k], p);
      uint64_t s = nodes[k].sub[i];
      if (s == 0)
        return;
      if (s & 1)
      {
        Node nn;
        int xb = i & 1, yb = (i & 2) / 2, zb = (i & 4) / 4;
        nn.c = V3{nodes[k].c.x + (2 * xb - 1) * nodes[k].side / 4, nodes[k].c.y + (2 * yb - 1) * nodes[k].side / 4,
                  nodes[k].c.z + (2 * zb - 1) * nodes[k].side / 4};
        nn.side = nodes[k].side / 2;
        for (int j = 0; j < 8; j++)
          nn.sub[j] = 0;
        nn.sub[octant(nn, p)] = s;
        nodes.push_back(nn);
        nodes[k].sub[i] = (uint64_t)(nodes.size() - 1) << 1;
        return;
      }
      k = s >> 1;
    }
  }
  bool blockPut(int64_t b, uint32_t id)
  {
    std::vector<uint32_t> &v = blocks[b];
    std::vector<V3> &w = bloc[b];
    std::vector<uint16_t> &ht = bhash[b];
    if (ht.empty())
      ht.assign(kHash, 0);
    const V3 p = loc[id];
    uint32_t h = hashOf(p) & (kHash - 1);
    for (; ht[h]; h = (h + 1) & (kHash - 1))
    {
      const V3 &q = w[ht[h] - 1];
      if (q.x == p.x && q.y == p.y && q.z == p.z)
      {
        v[ht[h] - 1] = id;   // last one wins
        return true;
      }
    }
    if ((int)v.size() < kRecords)
    {
      v.push_back(id);
      w.push_back(p);
      ht[h] = (uint16_t)w.size();
      return true;
    }
    return false;
  }
  void put(uint32_t id)
  {
    const V3 &p = loc[id];
    if (std::isnan(p.x) || std::isnan(p.y) || std::isnan(p.z))
      return;
    int64_t b = findBlock(p);
    if (b < 0)
    {
      b = (int64_t)blocks.size();
      blocks.emplace_back();
      bloc.emplace_back();
      bhash.emplace_back();
      setBlock(p, b);
    }
    if (!blockPut(b, id))
    {
      std::vector<uint32_t> moved;
      moved.swap(blocks[b]);
      bloc[b].clear();
      bhash[b].assign(kHash, 0);
      splitAt(p);
      for (uint32_t m : moved)
        spill.push_back(m);
      b = findBlock(p);
      blockPut(b, id);
    }
  }
  void drain()
  {
    while (!spill.empty())
    {
      uint32_t id = spill.back();
      spill.pop_back();
      put(id);
    }
  }
  void findBlocks(size_t k, const Shape &sh, const CubeR &cube, std::vector<int64_t> &out) const
  {
    if (!sh.meets(cube))
      return;
    for (int i = 0; i < 8; i++)
    {
      uint64_t s = nodes[k].sub[i];
      if (s & 1)
      {
        if (sh.meets(octCube(nodes[k], i)))
          out.push_back((int64_t)(s >> 1));
      }
      else if (s)
        findBlocks(s >> 1, sh, octCube(nodes[k], i), out);
    }
  }
  /* OctStore::pointsIn (octree.cpp:1214-1242) */
  void pointsIn(const Shape &sh, std::vector<uint32_t> &out) const
  {
    std::vector<int64_t> bl;
    findBlocks(0, sh, CubeR{nodes[0].c, nodes[0].side}, bl);
    CubeR cube{V3{0, 0, 0}, 0};
    out.clear();
    for (int64_t b : bl)
    {
      const std::vector<uint32_t> &v = blocks[b];
      if (v.size())
        cube = findCube(loc[v[0]]);
      if (sh.inCube(cube))
        out.insert(out.end(), v.begin(), v.end());
      else
        for (uint32_t id : v)
          if (sh.in(loc[id]))
            out.push_back(id);
    }
  }
  void dfsLeaves(size_t k, std::vector<std::pair<CubeR, int64_t>> &out) const
  {
    for (int i = 0; i < 8; i++)
    {
      uint64_t s = nodes[k].sub[i];
      if (s & 1)
        out.push_back({octCube(nodes[k], i), (int64_t)(s >> 1)});
      else if (s)
        dfsLeaves(s >> 1, out);
    }
  }
};

/* Octree::sizeFit (octree.cpp:268-310) */
void sizeFitR(const V3 &mn, const V3 &mx, V3 &center, double &side)
{
  double minx = std::min(mn.x, mx.x), maxx = std::max(mn.x, mx.x);
  double miny = std::min(mn.y, mx.y), maxy = std::max(mn.y, mx.y);
  double minz = std::min(mn.z, mx.z), maxz = std::max(mn.z, mx.z);
  center = V3{0, 0, 0};
  if (maxz <= minz && maxy <= miny && maxx <= minx)
  {
    side = 0;
    return;
  }
  int e;
  side = (maxx + maxy + maxz - minx - miny - minz) / 3;
  side /= frexp(side, &e) * 2;
  double x = minx - side, y = miny - side, z = minz - side;
  while (x + side <= maxx || y + side <= maxy || z + side <= maxz)
  {
    side *= 2;
    x = (rint((minx + maxx) / side * 8) - 8) * side / 16;
    y = (rint((miny + maxy) / side * 8) - 8) * side / 16;
    z = (rint((minz + maxz) / side * 8) - 8) * side / 16;
  }
  center = V3{x + side / 2, y + side / 2, z + side / 2};
}

/* ---------------- flowsnake tiling (flowsnake.cpp, eisenstein.cpp) ---------------- */

const double kSquareSides[12] = {
  0.6583539906808145, 1.8501627472990723, 4.286014912881196, 12.6716160058597,
  32.85016274729906, 79.01914481623778, 243.0343734125204, 592.8501627472989,
  1510.850162747299, 4399.956311577825, 10731.850162747294, 29198.8501627473};
const int kLoLim[12] = {0, -4, -18, -214, -900, -10504, -44118, -514714, -24242424, -25221004, -105928218, -1235829214};
const int kHiLim[12] = {0, 2, 30, 128, 1500, 6302, 73530, 308828, 3603000, 15132602, 176547030, 741497528};
const unsigned char kFlowTable[6][7] = {
  {0x52, 0x05, 0x06, 0x24, 0x33, 0x40, 0x01},
  {0x31, 0x10, 0x12, 0x05, 0x43, 0x54, 0x16},
  {0x46, 0x24, 0x21, 0x10, 0x53, 0x35, 0x22},
  {0x31, 0x10, 0x03, 0x54, 0x36, 0x35, 0x22},
  {0x46, 0x24, 0x13, 0x35, 0x42, 0x40, 0x01},
  {0x52, 0x05, 0x23, 0x40, 0x51, 0x54, 0x16}};

struct Eis
{
  int x, y;
};
Eis emul(Eis a, Eis b) { return Eis{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x - a.y * b.y}; }

int permuteDigits(int n)
{
  int dig[11], state = 0;
  n += 1235829214;
  for (int i = 0; i < 11; i++)
  {
    dig[i] = n % 7;
    n /= 7;
  }
  n = 0;
  for (int i = 10; i >= 0; i--)
  {
    int t = kFlowTable[state][dig[i]];
    state = t >> 4;
    n = 7 * n + (t & 7);
  }
  return n - 988663371;
}

Eis centredBase7ToEis(int n)
{
  Eis ret{0, 0}, pw{1, 0};
  const Eis base{2, -1};
  while (n)
  {
    int d = n % 7;
    if (d > 3)
      d -= 7;
    if (d < -3)
      d += 7;
    n = (n - d) / 7;
    int yy = (d + 4) / 3 - 1;
    Eis dg{d - 2 * yy, yy};
    Eis t = emul(dg, pw);
    ret.x += t.x;
    ret.y += t.y;
    pw = emul(pw, base);
  }
  return ret;
}

Eis toFlowsnakeR(int n) { return centredBase7ToEis(permuteDigits(n)); }

struct Snake
{
  V3 center;
  double spacing;
  int idx, lo, hi;
  void setSize(const CubeR &cube, double desired)
  {
    double best = INFINITY;
    idx = 0;
    for (int i = 0; i < 12; i++)
    {
      double sp = cube.side / kSquareSides[i];
      double diff = fabs(log(sp / desired));
      if (diff < best)
      {
        best = diff;
        idx = i;
      }
    }
    center = cube.c;
    spacing = cube.side / kSquareSides[idx];
    lo = kLoLim[idx];
    hi = kHiLim[idx];
  }
  CylinderR cyl(Eis e) const
  {
    double rad = spacing * 41 / 71;
    double re = (e.x - e.y / 2.) * spacing, im = (e.y * kSqrt34) * spacing;
    return CylinderR(re + center.x, im + center.y, rad);
  }
};

/* BoundRect over the two header corners (boundrect.cpp:44-58, point.cpp dirbound) */
CubeR snakeCube(const V3 &a, const V3 &b)
{
  double bounds[6];
  for (int i = 0; i < 6; i++)
    bounds[i] = INFINITY;
  const V3 pts[2] = {a, b};
  for (const V3 &p : pts)
  {
    for (int i = 0; i < 4; i++)
    {
      int ang = i * kDeg90;
      double nb = p.x * cosInt(ang) + p.y * sinInt(ang);
      if (nb < bounds[i])
        bounds[i] = nb;
    }
    if (p.z < bounds[4])
      bounds[4] = p.z;
    if (-p.z < bounds[5])
      bounds[5] = -p.z;
  }
  double left = bounds[0], bottom = bounds[1], right = -bounds[2], top = -bounds[3];
  double low = bounds[4], high = -bounds[5];
  double side = right - left;
  if (top - bottom > side)
    side = top - bottom;
  if (high - low > side)
    side = high - low;
  return CubeR{V3{(right + left) / 2, (top + bottom) / 2, (high + low) / 2}, side};
}

/* ---------------- tiles, scan, postscan, classify ---------------- */

struct TileR
{
  int nPoints = 0, nGround = 0, treeFlags = 0;
  double density = 0, hScan = 0, h = 0, height = 0;
};

struct Pipeline
{
  Store st;
  Snake snake;
  std::vector<Eis> order;
  std::unordered_map<int64_t, int> addrToK;   // Eisenstein -> flowsnake position
  std::vector<TileR> tiles;
  wbo_params prm;

  static int64_t akey(Eis e) { return ((int64_t)e.x << 32) ^ (uint32_t)e.y; }
  const TileR *tileAt(Eis e) const
  {
    auto it = addrToK.find(akey(e));
    return it == addrToK.end() ? nullptr : &tiles[it->second];
  }

  /* scanCylinder (scan.cpp:31-140) */
  void scanTile(size_t k)
  {
    CylinderR cyl = snake.cyl(order[k]);
    std::vector<uint32_t> pts;
    st.pointsIn(cyl, pts);
    if (pts.empty())
      return;
    size_t n = pts.size();
    std::vector<double> px(n), py(n), pz(n);
    for (size_t i = 0; i < n; i++)
    {
      const V3 &p = st.loc[pts[i]];
      px[i] = p.x - cyl.cx;
      py[i] = p.y - cyl.cy;
      pz[i] = p.z - 0.0;
    }
    double sl[3];
    lsqPlane(px.data(), py.data(), pz.data(), (unsigned)n, sl);
    double sx = sl[0], sy = sl[1];
    double len = hypotR(sx, sy);
    if (len > 1)
    {
      sx /= len;
      sy /= len;
    }
    if (std::isnan(sx) || std::isnan(sy))
      sx = sy = 0;
    double bottom = INFINITY, bottom2 = INFINITY, top = -INFINITY;
    std::vector<double> uz(n);
    for (size_t i = 0; i < n; i++)
    {
      double z = sy * py[i] + sx * px[i];
      uz[i] = pz[i] - z;
      if (uz[i] < bottom)
      {
        bottom2 = bottom;
        bottom = uz[i];
      }
      if (uz[i] > top)
        top = uz[i];
    }
    if (std::isinf(bottom2))
      bottom2 = bottom;
    int histo[7] = {0, 0, 0, 0, 0, 0, 0};
    size_t nBottom = 0;
    for (size_t i = 0; i < n; i++)
      if (uz[i] < bottom2 + 2 * cyl.r)
      {
        nBottom++;
        int sector = (int)lrint(atan2(py[i], px[i]) * 3 / M_PI);
        if (sector < 0)
          sector += 6;
        sector = (sector % 6) + 1;
        if (hypotR(px[i], py[i]) < cyl.r / kSqrt7)
          sector = 0;
        histo[sector]++;
      }
    double density = 0;
    int treeFlags = 0;
    for (int i = 0; i < 7; i++)
      density += sq(histo[i]);
    if (n > nBottom && density < 7)
      treeFlags = 1;
    density = sqrt(density) * kSqrt7 / sq(cyl.r) / M_PI;
    if (n > nBottom && density < 0.5)
      treeFlags = 1;
    if (top - bottom > 1.5)
      treeFlags = 1;
    TileR &t = tiles[k];
    t.nPoints = (int)n;
    t.nGround = 0;
    t.density = density;
    t.treeFlags = treeFlags;
    t.h = t.hScan = sqrt(1 / density + sq(prm.min_hyp_size));
    t.height = top - bottom;
  }

  /* Tiles scanned on demand in a sampled run (each exactly once). */
  std::vector<std::once_flag> *scanOnce = nullptr;
  std::atomic<uint64_t> nScanned{0};
  void ensureScanned(size_t k)
  {
    if (scanOnce)
      std::call_once((*scanOnce)[k], [&] {
        scanTile(k);
        nScanned++;
      });
  }
  const TileR *tileAtScanned(Eis e)
  {
    auto it = addrToK.find(akey(e));
    if (it == addrToK.end())
      return nullptr;
    ensureScanned((size_t)it->second);
    return &tiles[it->second];
  }

  /* postscanCylinder (scan.cpp:142-179) */
  double postscanTile(size_t k)
  {
    const TileR &me = tiles[k];
    if (!me.nPoints)
      return me.h;
    static const Eis ring[6] = {{1, 0}, {1, 1}, {0, 1}, {-1, 0}, {-1, -1}, {0, -1}};
    int i = 1, count = 0, nontree, ringcount;
    do
    {
      nontree = ringcount = 0;
      for (int j = 0; j < 6 && (me.treeFlags & 1); j++)
      {
        Eis a{order[k].x + ring[j].x * i, order[k].y + ring[j].y * i};
        const TileR *t = tileAtScanned(a);
        if (t && t->nPoints)
        {
          ringcount++;
          if (t->treeFlags & 1)
            count++;
          else
            nontree++;
        }
      }
      ++i;
    } while (ringcount && !nontree);
    return sqrt(sq(me.h) + sq(count * snake.spacing / 6));
  }

  /* surround (classify.cpp:67-94) */
  static bool surround(std::set<int> &dirs)
  {
    int n = 0, first = 0, last = 0, penult = 0;
    const int parity = 0;
    bool ret = dirs.size() > 1;
    std::vector<int> delenda;
    for (auto it = dirs.begin(); it != dirs.end(); ++it, ++n)
    {
      if (it == dirs.begin())
        first = *it;
      else if ((((unsigned)*it - (unsigned)last) & INT_MAX) >= (unsigned)kDeg144)
        ret = false;
      if ((n & 1) == parity && n > 1 && (((unsigned)*it - (unsigned)last) & INT_MAX) < (unsigned)kDeg30 &&
          (((unsigned)last - (unsigned)penult) & INT_MAX) < (unsigned)kDeg30)
        delenda.push_back(last);
      penult = last;
      last = *it;
    }
    if ((((unsigned)first - (unsigned)last) & INT_MAX) >= (unsigned)kDeg144)
      ret = false;
    for (int d : delenda)
      dirs.erase(d);
    return ret;
  }

  /* Largest circular gap of a direction set (0 and twoDirs false below two). */
  static uint32_t largestGap(const std::set<int> &dirs, bool &twoDirs)
  {
    twoDirs = dirs.size() >= 2;
    if (!twoDirs)
      return 0;
    uint32_t worst = 0;
    int prev = *dirs.rbegin();
    for (int d : dirs)
    {
      worst = std::max(worst, ((uint32_t)d - (uint32_t)prev) & (uint32_t)INT_MAX);
      prev = d;
    }
    return worst;
  }

  /* classifyCylinder (classify.cpp:96-173): labels are returned, not stored;
     gaps (optional) receives each point's largest direction gap at the end of
     its loop (for a point that is not surrounded, that of all its neighbours)
     in degrees minus 144, 216 with fewer than two directions */
  void classifyTile(size_t k, std::vector<std::pair<uint32_t, uint8_t>> &res, int &nGround,
                    std::vector<double> *gaps = nullptr) const
  {
    CylinderR cyl = snake.cyl(order[k]);
    std::vector<uint32_t> cp;
    st.pointsIn(cyl, cp);
    res.clear();
    nGround = 0;
    if (cp.empty())
      return;
    std::sort(cp.begin(), cp.end(), [&](uint32_t a, uint32_t b) { return st.loc[a].z < st.loc[b].z; });
    const TileR &t = tiles[k];
    std::vector<uint32_t> down;
    for (uint32_t id : cp)
    {
      const V3 &p = st.loc[id];
      std::set<int> dirs;
      bool above = false;
      HyperboloidR hyp(V3{p.x - 0, p.y - 0, p.z - prm.thickness}, t.h, prm.max_slope);
      for (size_t j = 0; j < down.size() && !above; j++)
      {
        const V3 &q = st.loc[down[j]];
        if (hyp.in(q) && hypotR(p.x - q.x, p.y - q.y) != 0)
          dirs.insert(atan2iR(q.y - p.y, q.x - p.x));
        if (surround(dirs))
          above = true;
      }
      if (!above)
        st.pointsIn(hyp, down);
      // dirsP: the directions of pointsIn(hyp) alone.  The first loop above
      // can add a point the hyperboloid holds but pointsIn leaves out (one
      // outside the root cube whose block the shape does not meet) when the
      // previous point's list had it; the margin reports the pointsIn set's gap.
      std::set<int> dirsP;
      const bool secondLoop = !above;
      for (size_t j = 0; j < down.size() && !above; j++)
      {
        const V3 &q = st.loc[down[j]];
        if (hypotR(p.x - q.x, p.y - q.y) != 0)
        {
          int d = atan2iR(q.y - p.y, q.x - p.x);
          dirs.insert(d);
          if (gaps)
            dirsP.insert(d);
        }
        if (surround(dirs))
          above = true;
      }
      res.push_back({id, (uint8_t)(above ? 1 : 2)});
      if (gaps)
      {
        bool two;
        uint32_t g = largestGap(secondLoop && !above ? dirsP : dirs, two);
        gaps->push_back(two ? ((double)g - (double)kDeg144) * (360.0 / 2147483648.0) : 216.0);
      }
      if (!above)
        nGround++;
    }
  }
};

/* Whether tile k is the last tile in flowsnake order whose cylinder holds the
 * point at p: only the six tiles around k can reach it (a cylinder's radius,
 * 41/71 of the spacing, is below the distance to the second ring minus that
 * radius). */
/* Whether OctStore::pointsIn(cyl) holds the stored point p (octree.cpp:
 * 1214-1242): its block must meet the cylinder, and then either the whole
 * block is taken (all eight corners inside) or the point itself is inside --
 * which differs from cyl.in(p) only for points outside the root cube. */
bool tileHolds(const Pipeline &P, size_t k, const V3 &p)
{
  const CylinderR cyl = P.snake.cyl(P.order[k]);
  const CubeR cube = P.st.findCube(p);
  if (!cyl.meets(cube))
    return false;
  return cyl.inCube(cube) || cyl.in(p);
}

bool ownsPoint(const Pipeline &P, size_t k, const V3 &p)
{
  static const Eis ring[6] = {{1, 0}, {1, 1}, {0, 1}, {-1, 0}, {-1, -1}, {0, -1}};
  for (const Eis &r : ring)
  {
    auto it = P.addrToK.find(Pipeline::akey(Eis{P.order[k].x + r.x, P.order[k].y + r.y}));
    if (it != P.addrToK.end() && (size_t)it->second > k && tileHolds(P, (size_t)it->second, p))
      return false;
  }
  return true;
}

Pipeline *gPipe = nullptr;

template <class F>
void parallelFor(size_t count, int threads, F f)
{
  std::atomic<size_t> next(0);
  auto work = [&]() {
    while (true)
    {
      size_t k = next.fetch_add(1);
      if (k >= count)
        break;
      f(k);
    }
  };
  if (threads <= 1)
  {
    work();
    return;
  }
  std::vector<std::thread> pool;
  for (int i = 0; i < threads; i++)
    pool.emplace_back(work);
  for (auto &t : pool)
    t.join();
}

struct SampleOut
{
  double tScan = 0, tClassify = 0;
  uint64_t nScanned = 0, nPoints = 0;
};

/* Scans, post-scans and (classify) classifies only the given tiles, scanning
 * the tiles their postscan reads on demand, from a fresh tile table; cls
 * (n entries) is zeroed and receives the class of every point a sampled tile
 * decides. */
SampleOut runSample(Pipeline &P, const int64_t *tiles, uint64_t count, int thr, uint8_t *cls, uint64_t n,
                    bool classify)
{
  SampleOut so;
  double t0 = nowSec();
  P.tiles.assign(P.order.size(), TileR());
  P.nScanned = 0;
  std::vector<size_t> smp;
  for (uint64_t i = 0; i < count; i++)
    if (tiles[i] >= 0 && (size_t)tiles[i] < P.order.size())
      smp.push_back((size_t)tiles[i]);
  std::vector<std::once_flag> once(P.order.size());
  P.scanOnce = &once;
  std::vector<double> hNew(smp.size());
  parallelFor(smp.size(), thr, [&](size_t i) {
    P.ensureScanned(smp[i]);
    hNew[i] = P.postscanTile(smp[i]);
  });
  for (size_t i = 0; i < smp.size(); i++)
    P.tiles[smp[i]].h = hNew[i];
  P.scanOnce = nullptr;
  double t1 = nowSec();
  so.tScan = t1 - t0;
  so.nScanned = P.nScanned.load();
  if (cls)
    memset(cls, 0, n);
  if (classify)
  {
    std::atomic<uint64_t> pts(0);
    parallelFor(smp.size(), thr, [&](size_t i) {
      size_t k = smp[i];
      std::vector<std::pair<uint32_t, uint8_t>> res;
      int ng = 0;
      P.classifyTile(k, res, ng);
      P.tiles[k].nGround = ng;
      pts += res.size();
      if (cls)
        for (auto &r : res)
          if (ownsPoint(P, k, P.st.loc[r.first]))
            cls[r.first] = r.second;
    });
    so.nPoints = pts.load();
    so.tClassify = nowSec() - t1;
  }
  return so;
}

}  // namespace

extern "C" {

void wbo_reset(void)
{
  delete gPipe;
  gPipe = nullptr;
}

int wbo_run(wbo_run_io *io, const wbo_params *p)
{
  ensureTables();
  wbo_reset();
  gPipe = new Pipeline;
  Pipeline &P = *gPipe;
  P.prm = *p;
  uint64_t n = io->n;
  P.st.loc.resize(n);
  for (uint64_t i = 0; i < n; i++)
  {
    V3 v{io->offset[0] + io->scale[0] * io->xyz[3 * i], io->offset[1] + io->scale[1] * io->xyz[3 * i + 1],
         io->offset[2] + io->scale[2] * io->xyz[3 * i + 2]};
    P.st.loc[i] = V3{v.x * io->unit, v.y * io->unit, v.z * io->unit};
  }
  V3 mn{io->minc[0] * io->unit, io->minc[1] * io->unit, io->minc[2] * io->unit};
  V3 mx{io->maxc[0] * io->unit, io->maxc[1] * io->unit, io->maxc[2] * io->unit};
  Node root;
  sizeFitR(mn, mx, root.c, root.side);
  for (int j = 0; j < 8; j++)
    root.sub[j] = 0;
  P.st.nodes.push_back(root);
  CubeR sc = snakeCube(mn, mx);
  P.snake.setSize(sc, p->tile_size);

  double t0 = nowSec();
  for (uint64_t i = 0; i < n; i++)
  {
    P.st.put((uint32_t)i);
    P.st.drain();
  }
  std::vector<std::vector<V3>>().swap(P.st.bloc);
  std::vector<std::vector<uint16_t>>().swap(P.st.bhash);
  if (io->canonical_order)
    for (auto &b : P.st.blocks)
      std::sort(b.begin(), b.end());
  double t1 = nowSec();

  std::vector<std::pair<CubeR, int64_t>> leaves;
  P.st.dfsLeaves(0, leaves);
  std::vector<int64_t> leafOfBlock(P.st.blocks.size(), -1);
  for (size_t i = 0; i < leaves.size(); i++)
    leafOfBlock[leaves[i].second] = (int64_t)i;
  if (io->block)
    for (uint64_t i = 0; i < n; i++)
      io->block[i] = -1;
  if (io->block_pos)
    for (uint64_t i = 0; i < n; i++)
      io->block_pos[i] = -1;
  if (io->leaf)
    for (uint64_t i = 0; i < n; i++)
      io->leaf[i] = -1;
  for (size_t b = 0; b < P.st.blocks.size(); b++)
    for (size_t j = 0; j < P.st.blocks[b].size(); j++)
    {
      uint32_t id = P.st.blocks[b][j];
      if (io->block)
        io->block[id] = (int64_t)b;
      if (io->block_pos)
        io->block_pos[id] = (int32_t)j;
      if (io->leaf)
        io->leaf[id] = leafOfBlock[b];
    }

  for (int k = P.snake.lo; k <= P.snake.hi; k++)
  {
    Eis e = toFlowsnakeR(k);
    P.addrToK[Pipeline::akey(e)] = (int)P.order.size();
    P.order.push_back(e);
  }
  P.tiles.assign(P.order.size(), TileR());
  int thr = io->threads > 0 ? io->threads : 1;
  double t2 = t1, t3 = t1, t4 = t1;
  io->n_scanned = 0;
  io->n_sample_points = 0;
  if (io->phases >= 2 && io->n_sample > 0)
  {
    SampleOut so = runSample(P, io->sample_tiles, io->n_sample, thr, io->cls, n, io->phases >= 3);
    t2 = t3 = t1 + so.tScan;
    t4 = t3 + so.tClassify;
    io->n_scanned = so.nScanned;
    io->n_sample_points = so.nPoints;
  }
  else if (io->phases >= 2)
  {
    parallelFor(P.order.size(), thr, [&](size_t k) { P.scanTile(k); });
    t2 = nowSec();
    std::vector<double> hNew(P.order.size());
    parallelFor(P.order.size(), thr, [&](size_t k) { hNew[k] = P.postscanTile(k); });
    for (size_t k = 0; k < P.order.size(); k++)
      P.tiles[k].h = hNew[k];
    t3 = nowSec();
  }
  if (io->cls && io->n_sample == 0)
    memset(io->cls, 0, n);
  if (io->phases >= 3 && io->n_sample == 0)
  {
    std::vector<std::atomic<int64_t>> best(n);
    for (uint64_t i = 0; i < n; i++)
      best[i].store(-1);
    // the margin of the tile that decides each point (the largest flowsnake
    // position that classified it), packed as (position + 1, float bits)
    std::vector<std::atomic<uint64_t>> mbest(io->margin ? n : 0);
    for (auto &m : mbest)
      m.store(0);
    parallelFor(P.order.size(), thr, [&](size_t k) {
      std::vector<std::pair<uint32_t, uint8_t>> res;
      std::vector<double> gaps;
      int ng = 0;
      P.classifyTile(k, res, ng, io->margin ? &gaps : nullptr);
      P.tiles[k].nGround = ng;
      if (io->margin)
        for (size_t q = 0; q < res.size(); q++)
        {
          float g = (float)gaps[q];
          uint32_t bits;
          memcpy(&bits, &g, 4);
          uint64_t v = ((uint64_t)(k + 1) << 32) | bits;
          std::atomic<uint64_t> &slot = mbest[res[q].first];
          uint64_t cur = slot.load();
          while (v > cur && !slot.compare_exchange_weak(cur, v))
          {
          }
        }
      for (auto &r : res)
      {
        int64_t v = ((int64_t)k << 8) | r.second;
        int64_t cur = best[r.first].load();
        while (v > cur && !best[r.first].compare_exchange_weak(cur, v))
        {
        }
      }
    });
    t4 = nowSec();
    if (io->cls)
      for (uint64_t i = 0; i < n; i++)
        if (best[i].load() >= 0)
          io->cls[i] = (uint8_t)(best[i].load() & 0xff);
    if (io->margin)
      for (uint64_t i = 0; i < n; i++)
      {
        uint64_t v = mbest[i].load();
        float g;
        uint32_t bits = (uint32_t)v;
        memcpy(&g, &bits, 4);
        io->margin[i] = v ? (double)g : NAN;
      }
  }
  io->n_blocks = P.st.blocks.size();
  io->n_leaves = leaves.size();
  io->n_tiles = P.order.size();
  io->root_center[0] = root.c.x;
  io->root_center[1] = root.c.y;
  io->root_center[2] = root.c.z;
  io->root_side = root.side;
  io->snake_center[0] = sc.c.x;
  io->snake_center[1] = sc.c.y;
  io->snake_center[2] = sc.c.z;
  io->snake_side = sc.side;
  io->spacing = P.snake.spacing;
  io->snake_index = P.snake.idx;
  io->t_build = t1 - t0;
  io->t_scan = t2 - t1;
  io->t_postscan = t3 - t2;
  io->t_classify = t4 - t3;
  return 0;
}

int wbo_sample(const int64_t *tiles, uint64_t count, int threads, uint8_t *cls, double *t_scan, double *t_classify,
               uint64_t *n_scanned, uint64_t *n_points)
{
  if (!gPipe)
    return -1;
  SampleOut so = runSample(*gPipe, tiles, count, threads > 0 ? threads : 1, cls, gPipe->st.loc.size(), true);
  if (t_scan)
    *t_scan = so.tScan;
  if (t_classify)
    *t_classify = so.tClassify;
  if (n_scanned)
    *n_scanned = so.nScanned;
  if (n_points)
    *n_points = so.nPoints;
  return 0;
}

int64_t wbo_points_in(int kind, const double *v, double r, double s, int sorted, uint32_t *out, uint64_t capacity)
{
  if (!gPipe)
    return -1;
  std::vector<uint32_t> ids;
  if (kind == 1)
    gPipe->st.pointsIn(CylinderR(v[0], v[1], r), ids);
  else if (kind == 2)
    gPipe->st.pointsIn(HyperboloidR(V3{v[0], v[1], v[2]}, r, s), ids);
  else
    return -1;
  if (sorted)   // stable: equal heights keep the unsorted order
    std::stable_sort(ids.begin(), ids.end(),
                     [&](uint32_t a, uint32_t b) { return gPipe->st.loc[a].z < gPipe->st.loc[b].z; });
  for (size_t i = 0; i < ids.size() && i < capacity; i++)
    out[i] = ids[i];
  return (int64_t)ids.size();
}

int64_t wbo_find_blocks(int kind, const double *v, double r, double s, int64_t *out, uint64_t capacity)
{
  if (!gPipe)
    return -1;
  std::vector<std::pair<CubeR, int64_t>> leaves;
  gPipe->st.dfsLeaves(0, leaves);
  std::vector<int64_t> leafOfBlock(gPipe->st.blocks.size(), -1);
  for (size_t i = 0; i < leaves.size(); i++)
    leafOfBlock[leaves[i].second] = (int64_t)i;
  std::vector<int64_t> bl;
  const Store &st = gPipe->st;
  CubeR root{st.nodes[0].c, st.nodes[0].side};
  if (kind == 1)
    st.findBlocks(0, CylinderR(v[0], v[1], r), root, bl);
  else if (kind == 2)
    st.findBlocks(0, HyperboloidR(V3{v[0], v[1], v[2]}, r, s), root, bl);
  else
    return -1;
  for (size_t i = 0; i < bl.size() && i < capacity; i++)
    out[i] = leafOfBlock[bl[i]];
  return (int64_t)bl.size();
}

int64_t wbo_snake_tiles(const double *minc, const double *maxc, double unit, double tile_size)
{
  ensureTables();
  V3 mn{minc[0] * unit, minc[1] * unit, minc[2] * unit};
  V3 mx{maxc[0] * unit, maxc[1] * unit, maxc[2] * unit};
  Snake sn;
  sn.setSize(snakeCube(mn, mx), tile_size);
  return (int64_t)sn.hi - sn.lo + 1;
}

int wbo_leaves(double *cs, int64_t *count)
{
  if (!gPipe)
    return -1;
  std::vector<std::pair<CubeR, int64_t>> leaves;
  gPipe->st.dfsLeaves(0, leaves);
  for (size_t i = 0; i < leaves.size(); i++)
  {
    cs[4 * i] = leaves[i].first.c.x;
    cs[4 * i + 1] = leaves[i].first.c.y;
    cs[4 * i + 2] = leaves[i].first.c.z;
    cs[4 * i + 3] = leaves[i].first.side;
    count[i] = (int64_t)gPipe->st.blocks[leaves[i].second].size();
  }
  return 0;
}

int wbo_tiles(wbo_tile *out)
{
  if (!gPipe)
    return -1;
  for (size_t k = 0; k < gPipe->order.size(); k++)
  {
    const TileR &t = gPipe->tiles[k];
    out[k] = wbo_tile{gPipe->order[k].x, gPipe->order[k].y, t.nPoints, t.nGround, t.treeFlags, 0,
                      t.density, t.hScan, t.h, t.height};
  }
  return 0;
}

void wbo_fill_tables(double *t, double *s, double *c)
{
  fillTables();
  memcpy(t, gTan, sizeof gTan);
  memcpy(s, gSin, sizeof gSin);
  memcpy(c, gCos, sizeof gCos);
}

void wbo_set_tables(const double *t, const double *s, const double *c)
{
  memcpy(gTan, t, sizeof gTan);
  memcpy(gSin, s, sizeof gSin);
  memcpy(gCos, c, sizeof gCos);
  gTablesSet = true;
}

int32_t wbo_atan2i(double y, double x)
{
  ensureTables();
  return atan2iR(y, x);
}

void wbo_atan2i_many(const double *yx, uint64_t n, int32_t *out)
{
  ensureTables();
  for (uint64_t i = 0; i < n; i++)
    out[i] = atan2iR(yx[2 * i], yx[2 * i + 1]);
}

void wbo_quadrant_trig(double *cs)
{
  int ang[4] = {0, kDeg90, kDeg180, kDeg270};
  for (int i = 0; i < 4; i++)
  {
    cs[2 * i] = cosInt(ang[i]);
    cs[2 * i + 1] = sinInt(ang[i]);
  }
}

double wbo_pairwisesum(const double *a, unsigned n) { return pairwise(a, n); }

void wbo_hypot_many(const double *ab, uint64_t n, double *out)
{
  for (uint64_t i = 0; i < n; i++)
    out[i] = hypotR(ab[2 * i], ab[2 * i + 1]);
}

void wbo_lsq_plane(const double *xyz, uint64_t rows, double *out3)
{
  std::vector<double> x(rows), y(rows), z(rows);
  for (uint64_t i = 0; i < rows; i++)
  {
    x[i] = xyz[3 * i];
    y[i] = xyz[3 * i + 1];
    z[i] = xyz[3 * i + 2];
  }
  lsqPlane(x.data(), y.data(), z.data(), (unsigned)rows, out3);
}

int wbo_hyperboloid_in(const double *v, double r, double s, const double *p)
{
  return HyperboloidR(V3{v[0], v[1], v[2]}, r, s).in(V3{p[0], p[1], p[2]});
}

int wbo_cylinder_in(const double *c, double r, const double *p)
{
  return CylinderR(c[0], c[1], r).in(V3{p[0], p[1], p[2]});
}

void wbo_size_fit(const double *mn, const double *mx, double *center3, double *side)
{
  V3 c;
  sizeFitR(V3{mn[0], mn[1], mn[2]}, V3{mx[0], mx[1], mx[2]}, c, *side);
  center3[0] = c.x;
  center3[1] = c.y;
  center3[2] = c.z;
}

int wbo_flowsnake_limits(int idx, int32_t *lo, int32_t *hi)
{
  if (idx < 0 || idx > 11)
    return -1;
  *lo = kLoLim[idx];
  *hi = kHiLim[idx];
  return 0;
}

void wbo_flowsnake(int idx, int32_t *exy)
{
  for (int k = kLoLim[idx], j = 0; k <= kHiLim[idx]; k++, j++)
  {
    Eis e = toFlowsnakeR(k);
    exy[2 * j] = e.x;
    exy[2 * j + 1] = e.y;
  }
}

}  // extern "C"

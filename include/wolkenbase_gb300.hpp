/* wolkenbase_gb300.hpp -- header-only C++ adapter over the C ABI of
 * wolkenbase_gb300.h that keeps the call shapes of the reference's octree,
 * point store and stage entry points, so wolkenbase's own C++ can switch a
 * phase to the GPU without changing its callers:
 *
 *   reference (phma/wolkenbase)                      here (namespace wolkenbase_gb300)
 *   octRoot.sizeFit + octStore.put per point         OctStore::put(wb_cloud) for the whole block
 *     (octree.cpp:268-310, 849-876; TH_READ)
 *   Octree::findBlock(xyz)        (octree.h:61)      OctStore::findBlock(p)        any p with getx/gety/getz
 *   Octree::findBlocks(Shape)     (octree.h:63)      OctStore::findBlocks(Cylinder | Hyperboloid)
 *   OctStore::pointsIn(Shape,sorted) (octree.h:177)  OctStore::pointsIn(Cylinder | Hyperboloid, sorted)
 *   OctStore::getNumBlocks()      (octree.h:162)     OctStore::getNumBlocks()
 *   OctStore::getAll(block)       (octree.h:171)     OctStore::getAll(block)
 *   OctStore::countClasses()      (octree.h:111)     OctStore::countClasses()
 *   OctStore::countClasses(block) (octree.h:170)     OctStore::countClasses(block)
 *   scanCylinder / postscanCylinder per tile         scanCylinders(store, params) over every tile
 *     (scan.h:27-28; TH_SCAN, TH_POSTSCAN)
 *   classifyCylinder per tile (classify.h:24;        classifyCylinders(store, params, cls) over every tile
 *     TH_SPLIT)
 *   tiles[Eisenstein] (tile.cpp:27)                  tiles(store), tileAt(store, e)
 *
 * Points travel as record indices into the caller's LAS point block (the
 * reference copies LasPoint values); blocks are numbered depth-first (the
 * reference numbers them in insertion order, which depends on thread timing).
 * Shapes are given by the arguments the reference constructs them with
 * (Cylinder(xy, r), Hyperboloid(xyz, r, s)), since the reference's shape
 * classes keep their parameters private.  Errors throw wolkenbase_gb300::Error
 * carrying the WB_E* code.  Needs C++17 and libwolkenbase_gb300.so.
 */
#ifndef WOLKENBASE_GB300_HPP
#define WOLKENBASE_GB300_HPP
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>
#include "wolkenbase_gb300.h"

namespace wolkenbase_gb300
{

class Error : public std::runtime_error
{
public:
  Error(int code, const std::string &what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

private:
  int code_;
};

/* Classification settings with the reference's defaults (mainwindow.cpp:407-410). */
struct Params : wb_params
{
  Params(double tileSize = 1.0, double maxSlope = 1.0, double thick = 0.0, double minHypSize = 0.1)
  {
    tile_size = tileSize;
    max_slope = maxSlope;
    thickness = thick;
    min_hyp_size = minHypSize;
  }
};

/* Cylinder(xy c, double r) (shape.h, shape.cpp:207-218). */
struct Cylinder
{
  double cx, cy, r;
  Cylinder(double x, double y, double radius) : cx(x), cy(y), r(radius) {}
  template <class XY>
  Cylinder(XY c, double radius) : cx(c.getx()), cy(c.gety()), r(radius)
  {
  }
};

/* Hyperboloid(xyz v, double r, double s) (shape.h, shape.cpp:119-125). */
struct Hyperboloid
{
  double v[3], r, s;
  Hyperboloid(double x, double y, double z, double radius, double slope) : v{x, y, z}, r(radius), s(slope) {}
  template <class XYZ>
  Hyperboloid(XYZ vertex, double radius, double slope)
    : v{vertex.getx(), vertex.gety(), vertex.getz()}, r(radius), s(slope)
  {
  }
};

/* The point-record block of a LAS file as wb_cloud describes it, read from
 * the file's public header block (LAS 1.0-1.4).  LasHeader keeps the raw
 * scale and offset private, and its getScale()/getOffset() return them
 * multiplied by the unit, which would round differently from readPoint's
 * (offset + scale*X)*unit (las.cpp:808); the file holds the raw values. */
struct LasFileGeometry
{
  int pointFormat = 0;
  unsigned pointLength = 0;
  uint64_t pointOffset = 0, nPoints = 0;
  double scale[3] = {0, 0, 0}, offset[3] = {0, 0, 0}, minc[3] = {0, 0, 0}, maxc[3] = {0, 0, 0};
};

inline LasFileGeometry readLasGeometry(const std::string &fileName)
{
  std::ifstream f(fileName, std::ios::binary);
  unsigned char h[375];
  std::memset(h, 0, sizeof h);
  if (!f.read(reinterpret_cast<char *>(h), 227) || std::memcmp(h, "LASF", 4))
    throw Error(WB_EINVAL, "readLasGeometry: " + fileName + " is not a LAS file");
  f.read(reinterpret_cast<char *>(h) + 227, sizeof h - 227);   // LAS 1.4 fields, when present
  auto u16 = [&](int o) { return (unsigned)h[o] | (unsigned)h[o + 1] << 8; };
  auto u32 = [&](int o) { return (uint32_t)u16(o) | (uint32_t)u16(o + 2) << 16; };
  auto u64 = [&](int o) { return (uint64_t)u32(o) | (uint64_t)u32(o + 4) << 32; };
  auto f64 = [&](int o) {
    uint64_t b = u64(o);
    double d;
    std::memcpy(&d, &b, 8);
    return d;
  };
  LasFileGeometry g;
  const int minor = h[25];
  g.pointOffset = u32(96);
  g.pointFormat = h[104] & 0x3f;
  g.pointLength = u16(105);
  g.nPoints = u32(107);
  if (minor >= 4 && u64(247))
    g.nPoints = u64(247);
  for (int a = 0; a < 3; a++)
  {
    g.scale[a] = f64(131 + 8 * a);
    g.offset[a] = f64(155 + 8 * a);
    g.maxc[a] = f64(179 + 16 * a);
    g.minc[a] = f64(187 + 16 * a);
  }
  return g;
}

/* The wb_cloud of a point block read from a file with that geometry. */
inline wb_cloud cloudOf(const LasFileGeometry &g, const void *records, double unit)
{
  wb_cloud c;
  std::memset(&c, 0, sizeof c);
  c.records = records;
  c.n = g.nPoints;
  c.stride = g.pointLength;
  c.unit = unit;
  for (int a = 0; a < 3; a++)
  {
    c.scale[a] = g.scale[a];
    c.offset[a] = g.offset[a];
    c.minc[a] = g.minc[a];
    c.maxc[a] = g.maxc[a];
  }
  return c;
}

/* One cloud's octree and point store on the device (Octree octRoot +
 * OctStore octStore, octree.cpp:37-38). */
class OctStore
{
public:
  explicit OctStore(int device = 0, size_t hbmBudget = 0) : ctx_(wb_open(device, hbmBudget))
  {
    if (!ctx_)
      throw Error(WB_ECUDA, wb_last_error(nullptr));
  }
  ~OctStore() { wb_close(ctx_); }
  OctStore(const OctStore &) = delete;
  OctStore &operator=(const OctStore &) = delete;
  wb_ctx *context() const { return ctx_; }

  /* octRoot.sizeFit(header corners) + octStore.put of every record. */
  void put(const wb_cloud &cloud)
  {
    check(wb_octree_build(ctx_, &cloud));
    check(wb_synchronize(ctx_));
    n_ = cloud.n;
    first_.clear();
    count_.clear();
    order_.clear();
    cls_.clear();
  }

  int64_t findBlock(double x, double y, double z) const
  {
    const double p[3] = {x, y, z};
    int64_t leaf = -1;
    check(wb_octree_find_block(ctx_, p, 1, &leaf));
    return leaf;
  }
  template <class XYZ>
  int64_t findBlock(XYZ p) const
  {
    return findBlock(p.getx(), p.gety(), p.getz());
  }

  std::vector<int64_t> findBlocks(const Cylinder &c) const { return blocks(shape(c)); }
  std::vector<int64_t> findBlocks(const Hyperboloid &h) const { return blocks(shape(h)); }
  std::vector<uint32_t> pointsIn(const Cylinder &c, bool sorted = false) const { return points(shape(c), sorted); }
  std::vector<uint32_t> pointsIn(const Hyperboloid &h, bool sorted = false) const
  {
    return points(shape(h), sorted);
  }

  size_t getNumBlocks() const
  {
    wb_octree_stats s;
    check(wb_octree_info(ctx_, &s));
    return (size_t)s.n_leaves;
  }

  /* The block's points as record indices, in store order. */
  std::vector<uint32_t> getAll(int64_t block) const
  {
    table();
    if (block < 0 || (size_t)block >= first_.size())
      return {};
    return std::vector<uint32_t>(order_.begin() + first_[block], order_.begin() + first_[block] + count_[block]);
  }

  /* Stored points per class after classifyCylinders (all blocks). */
  std::map<int, size_t> countClasses() const
  {
    uint64_t t[256];
    check(wb_class_totals(ctx_, t));
    std::map<int, size_t> m;
    for (int k = 0; k < 256; k++)
      if (t[k])
        m[k] = (size_t)t[k];
    return m;
  }
  std::map<int, size_t> countClasses(int64_t block) const
  {
    std::map<int, size_t> m;
    for (uint32_t i : getAll(block))
      m[i < cls_.size() ? cls_[i] : 0]++;
    return m;
  }

private:
  friend void classifyCylinders(OctStore &, const Params &, std::vector<uint8_t> &, std::vector<float> *);
  wb_ctx *ctx_;
  uint64_t n_ = 0;
  mutable std::vector<uint32_t> first_, count_, order_;
  std::vector<uint8_t> cls_;

  void check(int rc) const
  {
    if (rc)
      throw Error(rc, wb_last_error(ctx_));
  }
  static wb_shape shape(const Cylinder &c)
  {
    wb_shape s;
    std::memset(&s, 0, sizeof s);
    s.kind = WB_SHAPE_CYLINDER;
    s.v[0] = c.cx;
    s.v[1] = c.cy;
    s.r = c.r;
    return s;
  }
  static wb_shape shape(const Hyperboloid &h)
  {
    wb_shape s;
    std::memset(&s, 0, sizeof s);
    s.kind = WB_SHAPE_HYPERBOLOID;
    for (int a = 0; a < 3; a++)
      s.v[a] = h.v[a];
    s.r = h.r;
    s.s = h.s;
    return s;
  }
  std::vector<int64_t> blocks(const wb_shape &s) const
  {
    uint64_t n = 0;
    int rc = wb_find_blocks(ctx_, &s, nullptr, 0, &n);
    if (rc && !(rc == WB_EINVAL && n))
      check(rc);
    std::vector<int64_t> out(n);
    check(wb_find_blocks(ctx_, &s, out.data(), n, &n));
    return out;
  }
  std::vector<uint32_t> points(const wb_shape &s, bool sorted) const
  {
    uint64_t n = 0;
    int rc = wb_points_in(ctx_, &s, sorted ? 1 : 0, nullptr, 0, &n);
    if (rc && !(rc == WB_EINVAL && n))
      check(rc);
    std::vector<uint32_t> out(n);
    check(wb_points_in(ctx_, &s, sorted ? 1 : 0, out.data(), n, &n));
    return out;
  }
  void table() const
  {
    if (!first_.empty())
      return;
    wb_octree_stats s;
    check(wb_octree_info(ctx_, &s));
    std::vector<double> cs(4 * s.n_leaves);
    first_.resize(s.n_leaves);
    count_.resize(s.n_leaves);
    order_.resize(s.n_distinct);
    check(wb_octree_leaves(ctx_, cs.data(), first_.data(), count_.data()));
    check(wb_octree_store_order(ctx_, order_.data()));
  }
};

/* TH_SCAN + TH_POSTSCAN: scanCylinder then postscanCylinder over every tile
 * in flowsnake order (scan.cpp:31-179). */
inline void scanCylinders(OctStore &st, const Params &p)
{
  int rc = wb_scan_tiles(st.context(), &p);
  if (rc == 0)
    rc = wb_synchronize(st.context());
  if (rc)
    throw Error(rc, wb_last_error(st.context()));
}

/* The tile table (Tile, tile.h:27-35) in flowsnake order. */
inline std::vector<wb_tile> tiles(const OctStore &st)
{
  uint64_t n = 0;
  int rc = wb_tiles(st.context(), nullptr, 0, &n);
  std::vector<wb_tile> out(n);
  if (rc == 0)
    rc = wb_tiles(st.context(), out.data(), n, &n);
  if (rc)
    throw Error(rc, wb_last_error(st.context()));
  return out;
}

/* tiles[e] for an Eisenstein address (any type with getx/gety); nullptr for
 * an address outside the flowsnake island. */
template <class E>
const wb_tile *tileAt(const std::vector<wb_tile> &table, E e)
{
  for (const wb_tile &t : table)
    if (t.ex == (int32_t)e.getx() && t.ey == (int32_t)e.gety())
      return &t;
  return nullptr;
}

/* TH_SPLIT: classifyCylinder over every tile (classify.cpp:96-173); the last
 * tile in flowsnake order that holds a point decides it.  cls has one entry
 * per record: on entry the record's class, on return 1 (not ground) or 2
 * (ground) wherever a tile holds the point.  margin (optional) receives each
 * record's decision margin in degrees (wb_classify_ex). */
inline void classifyCylinders(OctStore &st, const Params &p, std::vector<uint8_t> &cls,
                              std::vector<float> *margin = nullptr)
{
  cls.resize(st.n_);
  if (margin)
    margin->resize(st.n_);
  int rc = wb_classify_ex(st.context(), &p, cls.data(), 0, margin ? margin->data() : nullptr);
  if (rc)
    throw Error(rc, wb_last_error(st.context()));
  st.cls_ = cls;
}

}  // namespace wolkenbase_gb300
#endif

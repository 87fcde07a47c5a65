/* Headless serial driver over the reference's own hot-path sources.
 *
 * Test infrastructure only: this file is compiled together with the
 * reference's octree / scan / classify / flowsnake / angle sources (they stay
 * where they lie; oracle/Makefile names them) into oracle/_ref/wb_ref.  It is
 * used to pin the CPU restatement in oracle/wb_oracle.cpp and to write the
 * golden fixtures under tests/golden/.  Nothing in the product links it.
 *
 * The pipeline mode follows the reference's own serial flow:
 *   wolkentest.cpp:1076-1082   fillTanTables, startThreads(1) then stop
 *   wolkencanvas.cpp:497-520   octRoot.sizeFit(header corners), BoundRect cube,
 *                              snake.setSize(cube,tileSize), initTiles
 *   testpattern.cpp:43-54      octStore.put + drain of thread buffer 0
 *   threads.cpp:619-660        scanCylinder / postscanCylinder / classifyCylinder
 *                              over snake.next() in flowsnake order
 *   wolkencanvas.cpp:547-562   snake.restart and setIgnoreDupes between phases
 *
 * Modes (all binary I/O is little-endian, native layout):
 *   wb_ref pipeline IN OUT tileSize maxSlope thickness minHypSize [phases]
 *   wb_ref tables OUT                 atan2i tables (tanTable, sinTable, cosTable)
 *   wb_ref atan2i IN OUT              IN: n, then n pairs (y,x) doubles -> n int32
 *   wb_ref quadrant OUT               sin/cos(int) of 0, 90, 180, 270 degrees
 *   wb_ref flowsnake IDX OUT          toFlowsnake(n) for n in [loLim,hiLim]
 *   wb_ref lsq IN OUT                 linearLeastSquares on n x 3 systems
 *   wb_ref lasrw IN OUT FMT UNIT SX SY SZ X0 Y0 Z0 X1 Y1 Z1 CLS FIELDS SYSID
 *                                     LasHeader::readPoint of every record of
 *                                     the LAS file IN (fields -> FIELDS), class
 *                                     byte from CLS, writePoint into OUT opened
 *                                     as CloudOutput::openFiles opens a file
 *                                     (openWrite, setUnit, setScale, setVersion
 *                                     1.4, setPointFormat), then writeHeader
 *   wb_ref preview IN OUT X0 Y0 SIDE W H
 *                                     the octree built as in pipeline mode, then
 *                                     OctStore::countPointsIn and hiLoPointsIn of
 *                                     the Column of every pixel (uint64 count,
 *                                     double lo, double hi per pixel, row-major)
 *   wb_ref combine N S0x S0y S0z O0x O0y O0z ...   combineScales per axis
 *   wb_ref join F0 F1 ...             joinPointFormat
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <climits>
#include <chrono>
#include <string>
#include <vector>
#include <array>
#include <fstream>
#include <iostream>
#include <unistd.h>
#include "octree.h"
#include "scan.h"
#include "classify.h"
#include "flowsnake.h"
#include "tile.h"
#include "threads.h"
#include "angle.h"
#include "boundrect.h"
#include "leastsquares.h"
#include "manysum.h"
#include "las.h"
#include <new>

using namespace std;

extern double tanTable[511], cosTable[512], sinTable[512];
extern double minHyperboloidSize, maxSlope, thickness;
extern const int hiLim[], loLim[];

struct WbxyzHeader
{
  char magic[8];
  uint64_t n;
  double scale[3], offset[3], unit, minc[3], maxc[3];
};

static double nowSec()
{
  return chrono::duration<double>(chrono::steady_clock::now().time_since_epoch()).count();
}

static void die(const char *msg)
{
  fprintf(stderr, "wb_ref: %s\n", msg);
  exit(2);
}

static void startSerialStore(const string &dir)
{
  fillTanTables();
  startThreads(1);          // so that lockCube doesn't divide by 0
  waitForThreads(TH_STOP);
  joinThreads();
  octStore.open(dir + "/store.oct");
}

static void drainBuffer()
{
  LasPoint pnt;
  while (true)
  {
    pnt = debufferPoint(0);
    if (pnt.isEmpty())
      break;
    octStore.put(pnt);
  }
}

static int runPipeline(int argc, char **argv)
{
  if (argc < 8)
    die("pipeline IN OUT tileSize maxSlope thickness minHypSize [phases]");
  const char *inName = argv[2], *outName = argv[3];
  double tileSize = atof(argv[4]);
  maxSlope = atof(argv[5]);
  thickness = atof(argv[6]);
  minHyperboloidSize = atof(argv[7]);
  int phases = argc > 8 ? atoi(argv[8]) : 3;   // 1 build, 2 +scan/postscan, 3 +classify
  FILE *f = fopen(inName, "rb");
  if (!f) die("cannot open input");
  WbxyzHeader h;
  if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, "WBXYZ1", 6)) die("bad header");
  vector<int32_t> q(3 * h.n);
  if (h.n && fread(q.data(), 12, h.n, f) != h.n) die("short input");
  fclose(f);

  char tmpl[] = "/tmp/wbrefXXXXXX";
  char *dir = mkdtemp(tmpl);
  if (!dir) die("mkdtemp");
  startSerialStore(dir);

  vector<xyz> limits;
  xyz minc(h.minc[0] * h.unit, h.minc[1] * h.unit, h.minc[2] * h.unit);
  xyz maxc(h.maxc[0] * h.unit, h.maxc[1] * h.unit, h.maxc[2] * h.unit);
  limits.push_back(minc);
  limits.push_back(maxc);
  octRoot.sizeFit(limits);
  BoundRect br;
  br.include(minc);
  br.include(maxc);
  double side = br.right() - br.left();
  if (br.top() - br.bottom() > side) side = br.top() - br.bottom();
  if (br.high() - br.low() > side) side = br.high() - br.low();
  Cube cube(xyz((br.right() + br.left()) / 2, (br.top() + br.bottom()) / 2,
                (br.high() + br.low()) / 2), side);
  snake.setSize(cube, tileSize);
  initTiles();

  double t0 = nowSec();
  for (uint64_t i = 0; i < h.n; i++)
  {
    LasPoint p;
    p.location = xyz(h.offset[0] + h.scale[0] * q[3 * i], h.offset[1] + h.scale[1] * q[3 * i + 1],
                     h.offset[2] + h.scale[2] * q[3 * i + 2]) * h.unit;
    p.returnNum = 1;
    p.nReturns = 1;
    p.classification = 0;
    p.gpsTime = (double)i;
    octStore.put(p);
    drainBuffer();
  }
  double t1 = nowSec();

  int lo = 0, hi = -1;
  {
    // Recover the tile range the snake was sized to (same choice as Flowsnake::setSize).
    snake.restart();
    Eisenstein e = snake.next();
    (void)e;
  }
  vector<Eisenstein> order;
  snake.restart();
  while (true)
  {
    Eisenstein e = snake.next();
    if (e.getx() == INT_MIN) break;
    order.push_back(e);
  }
  vector<double> hScan(order.size(), 0.0);
  double t2 = t1, t3 = t1, t4 = t1;
  if (phases >= 2)
  {
    snake.restart();
    for (size_t k = 0; k < order.size(); k++)
      scanCylinder(snake.next());
    for (size_t k = 0; k < order.size(); k++)
      if (tiles.count(order[k]))
        hScan[k] = tiles[order[k]].hyperboloidSize;
    t2 = nowSec();
    snake.restart();
    for (size_t k = 0; k < order.size(); k++)
      postscanCylinder(snake.next());
    t3 = nowSec();
  }
  if (phases >= 3)
  {
    octStore.setIgnoreDupes(true);
    snake.restart();
    for (size_t k = 0; k < order.size(); k++)
      classifyCylinder(snake.next());
    t4 = nowSec();
  }

  // Per input point: block, position in block, class, leaf cube.
  uint64_t nb = octStore.getNumBlocks();
  vector<int64_t> blk(h.n, -1);
  vector<int32_t> pos(h.n, -1);
  vector<uint8_t> cls(h.n, 0);
  vector<double> leaf(4 * h.n, 0.0);
  for (uint64_t b = 0; b < nb; b++)
  {
    vector<LasPoint> pts = octStore.getAll(b);
    for (size_t j = 0; j < pts.size(); j++)
    {
      int64_t id = llrint(pts[j].gpsTime);
      if (id < 0 || (uint64_t)id >= h.n) die("bad gpsTime");
      blk[id] = b;
      pos[id] = (int32_t)j;
      cls[id] = (uint8_t)pts[j].classification;
      Cube c = octRoot.findCube(pts[j].location);
      leaf[4 * id] = c.getCenter().getx();
      leaf[4 * id + 1] = c.getCenter().gety();
      leaf[4 * id + 2] = c.getCenter().getz();
      leaf[4 * id + 3] = c.getSide();
    }
    octStore.disown();
  }
  FILE *o = fopen(outName, "wb");
  if (!o) die("cannot open output");
  uint64_t hdr[3] = {h.n, nb, (uint64_t)order.size()};
  fwrite(hdr, 8, 3, o);
  double geo[8] = {octRoot.getCenter().getx(), octRoot.getCenter().gety(), octRoot.getCenter().getz(),
                   octRoot.getSide(), cube.getCenter().getx(), cube.getCenter().gety(),
                   cube.getCenter().getz(), cube.getSide()};
  fwrite(geo, 8, 8, o);
  double sp = snake.getSpacing();
  fwrite(&sp, 8, 1, o);
  fwrite(blk.data(), 8, h.n, o);
  fwrite(pos.data(), 4, h.n, o);
  fwrite(cls.data(), 1, h.n, o);
  fwrite(leaf.data(), 8, 4 * h.n, o);
  for (size_t k = 0; k < order.size(); k++)
  {
    Eisenstein e = order[k];
    int32_t iv[6] = {e.getx(), e.gety(), 0, 0, 0, 0};
    double dv[4] = {0, 0, 0, 0};
    if (tiles.count(e))
    {
      Tile &t = tiles[e];
      iv[2] = t.nPoints;
      iv[3] = t.nGround;
      iv[4] = t.treeFlags;
      dv[0] = t.density;
      dv[1] = hScan[k];
      dv[2] = t.hyperboloidSize;
      dv[3] = t.height;
    }
    fwrite(iv, 4, 6, o);
    fwrite(dv, 8, 4, o);
  }
  fclose(o);
  printf("{\"n\": %llu, \"blocks\": %llu, \"tiles\": %zu, \"build_s\": %.6f, \"scan_s\": %.6f, "
         "\"postscan_s\": %.6f, \"classify_s\": %.6f}\n",
         (unsigned long long)h.n, (unsigned long long)nb, order.size(), t1 - t0, t2 - t1, t3 - t2, t4 - t3);
  string cmd = string("rm -rf ") + dir;
  if (system(cmd.c_str())) {}
  return 0;
}

static int runTables(int argc, char **argv)
{
  if (argc < 3) die("tables OUT");
  fillTanTables();
  FILE *o = fopen(argv[2], "wb");
  fwrite(tanTable, 8, 511, o);
  fwrite(sinTable, 8, 512, o);
  fwrite(cosTable, 8, 512, o);
  fclose(o);
  return 0;
}

static int runAtan2i(int argc, char **argv)
{
  if (argc < 4) die("atan2i IN OUT");
  fillTanTables();
  FILE *f = fopen(argv[2], "rb");
  uint64_t n;
  if (fread(&n, 8, 1, f) != 1) die("short");
  vector<double> yx(2 * n);
  if (fread(yx.data(), 16, n, f) != n) die("short");
  fclose(f);
  vector<int32_t> r(n);
  for (uint64_t i = 0; i < n; i++)
    r[i] = atan2i(yx[2 * i], yx[2 * i + 1]);
  FILE *o = fopen(argv[3], "wb");
  fwrite(r.data(), 4, n, o);
  fclose(o);
  return 0;
}

static int runQuadrant(int argc, char **argv)
{
  if (argc < 3) die("quadrant OUT");
  double v[8];
  int ang[4] = {0, DEG90, DEG180, DEG270};
  for (int i = 0; i < 4; i++)
  {
    v[2 * i] = cos(ang[i]);
    v[2 * i + 1] = sin(ang[i]);
  }
  FILE *o = fopen(argv[2], "wb");
  fwrite(v, 8, 8, o);
  fclose(o);
  return 0;
}

static int runFlowsnake(int argc, char **argv)
{
  if (argc < 4) die("flowsnake IDX OUT");
  int idx = atoi(argv[2]);
  FILE *o = fopen(argv[3], "wb");
  for (int n = loLim[idx]; n <= hiLim[idx]; n++)
  {
    Eisenstein e = toFlowsnake(n);
    int32_t v[2] = {e.getx(), e.gety()};
    fwrite(v, 4, 2, o);
  }
  fclose(o);
  return 0;
}

static int runLsq(int argc, char **argv)
{
  // IN: uint64 nsys; per system: uint64 rows, then rows*(x,y,1-col implied, z) as 3 doubles (x,y,z)
  if (argc < 4) die("lsq IN OUT");
  FILE *f = fopen(argv[2], "rb");
  FILE *o = fopen(argv[3], "wb");
  uint64_t ns;
  if (fread(&ns, 8, 1, f) != 1) die("short");
  for (uint64_t s = 0; s < ns; s++)
  {
    uint64_t rows;
    if (fread(&rows, 8, 1, f) != 1) die("short");
    vector<double> d(3 * rows);
    if (fread(d.data(), 24, rows, f) != rows) die("short");
    matrix a(rows, 3);
    vector<double> b;
    for (uint64_t i = 0; i < rows; i++)
    {
      a[i][0] = d[3 * i];
      a[i][1] = d[3 * i + 1];
      a[i][2] = 1;
      b.push_back(d[3 * i + 2]);
    }
    vector<double> x = linearLeastSquares(a, b);
    fwrite(x.data(), 8, 3, o);
  }
  fclose(f);
  fclose(o);
  return 0;
}

double combine1Scale(vector<double> &scales, vector<double> &offsets);

/* A LasHeader built in zeroed memory, so that the fields its constructor and
 * openWrite leave unset (source id, encoding, GUID, start of waveform data)
 * read as 0 in the header written. */
static LasHeader *zeroedHeader()
{
  void *mem = aligned_alloc(alignof(LasHeader), (sizeof(LasHeader) + alignof(LasHeader) - 1) / alignof(LasHeader) *
                                                    alignof(LasHeader));
  memset(mem, 0, sizeof(LasHeader));
  return new (mem) LasHeader;
}

static int runLasRW(int argc, char **argv)
{
  if (argc < 18) die("lasrw IN OUT FMT UNIT SX SY SZ X0 Y0 Z0 X1 Y1 Z1 CLS FIELDS SYSID");
  double unit = atof(argv[5]);
  xyz scale(atof(argv[6]), atof(argv[7]), atof(argv[8]));
  xyz lo(atof(argv[9]), atof(argv[10]), atof(argv[11])), hi(atof(argv[12]), atof(argv[13]), atof(argv[14]));
  LasHeader *in = zeroedHeader(), *out = zeroedHeader();
  in->setUnit(unit);
  in->openRead(argv[2]);
  size_t n = in->numberPoints();
  vector<unsigned char> cls(n);
  FILE *c = fopen(argv[15], "rb");
  if (!c || fread(cls.data(), 1, n, c) != n) die("classes");
  fclose(c);
  out->openWrite(argv[3], atoi(argv[17]));
  out->setUnit(unit);
  out->setScale(lo, hi, scale);
  out->setVersion(1, 4);
  out->setPointFormat(atoi(argv[4]));
  FILE *f = fopen(argv[16], "wb");
  for (size_t i = 0; i < n; i++)
  {
    LasPoint p = in->readPoint(i);
    double xyzv[3] = {p.location.getx(), p.location.gety(), p.location.getz()};
    uint8_t sd = p.scanDirection, el = p.edgeLine;
    int32_t ang = p.scanAngle;
    fwrite(xyzv, 8, 3, f);
    fwrite(&p.intensity, 2, 1, f);
    fwrite(&p.returnNum, 2, 1, f);
    fwrite(&p.nReturns, 2, 1, f);
    fwrite(&sd, 1, 1, f);
    fwrite(&el, 1, 1, f);
    fwrite(&p.classification, 2, 1, f);
    fwrite(&p.classificationFlags, 2, 1, f);
    fwrite(&p.scannerChannel, 2, 1, f);
    fwrite(&p.userData, 2, 1, f);
    fwrite(&ang, 4, 1, f);
    fwrite(&p.pointSource, 2, 1, f);
    fwrite(&p.gpsTime, 8, 1, f);
    fwrite(&p.red, 2, 1, f);
    fwrite(&p.green, 2, 1, f);
    fwrite(&p.blue, 2, 1, f);
    fwrite(&p.nir, 2, 1, f);
    p.classification = cls[i];
    out->writePoint(p);
  }
  fclose(f);
  out->writeHeader();
  out->close();
  in->close();
  return 0;
}

static int runPreview(int argc, char **argv)
{
  if (argc < 9)
    die("preview IN OUT X0 Y0 SIDE W H");
  FILE *f = fopen(argv[2], "rb");
  if (!f) die("cannot open input");
  WbxyzHeader h;
  if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, "WBXYZ1", 6)) die("bad header");
  vector<int32_t> q(3 * h.n);
  if (h.n && fread(q.data(), 12, h.n, f) != h.n) die("short input");
  fclose(f);
  const double x0 = atof(argv[4]), y0 = atof(argv[5]), side = atof(argv[6]);
  const int w = atoi(argv[7]), hgt = atoi(argv[8]);
  char tmpl[] = "/tmp/wbrefXXXXXX";
  char *dir = mkdtemp(tmpl);
  if (!dir) die("mkdtemp");
  startSerialStore(dir);
  vector<xyz> limits;
  limits.push_back(xyz(h.minc[0] * h.unit, h.minc[1] * h.unit, h.minc[2] * h.unit));
  limits.push_back(xyz(h.maxc[0] * h.unit, h.maxc[1] * h.unit, h.maxc[2] * h.unit));
  octRoot.sizeFit(limits);
  for (uint64_t i = 0; i < h.n; i++)
  {
    LasPoint p;
    p.location = xyz(h.offset[0] + h.scale[0] * q[3 * i], h.offset[1] + h.scale[1] * q[3 * i + 1],
                     h.offset[2] + h.scale[2] * q[3 * i + 2]) * h.unit;
    p.returnNum = 1;
    p.nReturns = 1;
    p.gpsTime = (double)i;
    octStore.put(p);
    drainBuffer();
  }
  FILE *o = fopen(argv[3], "wb");
  if (!o) die("cannot open output");
  for (int j = 0; j < hgt; j++)
    for (int i = 0; i < w; i++)
    {
      Column col(xy(x0 + i * side, y0 + j * side), side);
      uint64_t cnt = octStore.countPointsIn(col);
      array<double, 2> hl = octStore.hiLoPointsIn(col);
      octStore.disown();
      fwrite(&cnt, 8, 1, o);
      fwrite(&hl[0], 8, 1, o);
      fwrite(&hl[1], 8, 1, o);
    }
  fclose(o);
  string cmd = string("rm -rf ") + dir;
  if (system(cmd.c_str())) {}
  return 0;
}

static int runCombine(int argc, char **argv)
{
  if (argc < 3) die("combine N S O ...");
  int n = atoi(argv[2]);
  if (argc < 3 + 6 * n) die("combine: 6 numbers per file");
  for (int k = 0; k < 3; k++)
  {
    vector<double> s, o;
    for (int i = 0; i < n; i++)
    {
      s.push_back(atof(argv[3 + 6 * i + k]));
      o.push_back(atof(argv[3 + 6 * i + 3 + k]));
    }
    printf("%.17g\n", combine1Scale(s, o));
  }
  return 0;
}

static int runJoin(int argc, char **argv)
{
  vector<int> f;
  for (int i = 2; i < argc; i++)
    f.push_back(atoi(argv[i]));
  printf("%d\n", joinPointFormat(f));
  return 0;
}

int main(int argc, char **argv)
{
  if (argc < 2) die("mode required");
  string mode = argv[1];
  if (mode == "pipeline") return runPipeline(argc, argv);
  if (mode == "tables") return runTables(argc, argv);
  if (mode == "atan2i") return runAtan2i(argc, argv);
  if (mode == "quadrant") return runQuadrant(argc, argv);
  if (mode == "flowsnake") return runFlowsnake(argc, argv);
  if (mode == "lsq") return runLsq(argc, argv);
  if (mode == "lasrw") return runLasRW(argc, argv);
  if (mode == "preview") return runPreview(argc, argv);
  if (mode == "combine") return runCombine(argc, argv);
  if (mode == "join") return runJoin(argc, argv);
  die("unknown mode");
  return 2;
}

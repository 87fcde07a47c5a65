/* Host-side geometry set-up: octree root, tile grid, flowsnake tile order.
 *
 * These run once per cloud on the host, as in the reference, and fix the
 * numbers every kernel works against:
 *   Octree::sizeFit          octree.cpp:268-310
 *   BoundRect cube           wolkencanvas.cpp:501-518, boundrect.cpp:44-58
 *   Flowsnake::setSize       flowsnake.cpp:208-229
 *   toFlowsnake              flowsnake.cpp:92-136 (iToFlowsnake + baseFlow)
 * The flowsnake tables (island sizes, counter ranges and the digit-state
 * table of the Gosper curve) are the reference's data: the tile order and
 * tile spacing must be the same for the classification to be the same.
 */
#include <cmath>
#include <vector>
#include <cstdint>
#include "wb_internal.h"
#include "angle_tables.h"

namespace
{
const double kSquareSides[12] = {
  0.6583539906808145, 1.8501627472990723, 4.286014912881196, 12.6716160058597,
  32.85016274729906, 79.01914481623778, 243.0343734125204, 592.8501627472989,
  1510.850162747299, 4399.956311577825, 10731.850162747294, 29198.8501627473};
const int kLoLim[12] = {0, -4, -18, -214, -900, -10504, -44118, -514714, -24242424, -25221004, -105928218,
                        -1235829214};
const int kHiLim[12] = {0, 2, 30, 128, 1500, 6302, 73530, 308828, 3603000, 15132602, 176547030, 741497528};
const unsigned char kStateTable[6][7] = {
  {0x52, 0x05, 0x06, 0x24, 0x33, 0x40, 0x01},
  {0x31, 0x10, 0x12, 0x05, 0x43, 0x54, 0x16},
  {0x46, 0x24, 0x21, 0x10, 0x53, 0x35, 0x22},
  {0x31, 0x10, 0x03, 0x54, 0x36, 0x35, 0x22},
  {0x46, 0x24, 0x13, 0x35, 0x42, 0x40, 0x01},
  {0x52, 0x05, 0x23, 0x40, 0x51, 0x54, 0x16}};

struct E2
{
  long long x, y;
};

E2 mulE(E2 a, E2 b) { return E2{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x - a.y * b.y}; }

/* Counter -> centred base-7 number along the curve: the digits are read most
 * significant first through the six-state replacement table. */
int curveDigits(int n)
{
  int dig[11], state = 0;
  n += 1235829214;
  for (int i = 0; i < 11; i++)
  {
    dig[i] = n % 7;
    n /= 7;
  }
  int r = 0;
  for (int i = 10; i >= 0; i--)
  {
    int t = kStateTable[state][dig[i]];
    state = t >> 4;
    r = 7 * r + (t & 7);
  }
  return r - 988663371;
}

/* Centred base-7 number -> Eisenstein integer in base 2-w (digit d maps to
 * x = d - 2y, y = (d+4)/3 - 1). */
E2 toEisenstein(int n)
{
  E2 acc{0, 0}, pw{1, 0};
  const E2 base{2, -1};
  while (n)
  {
    int d = n % 7;
    if (d > 3)
      d -= 7;
    if (d < -3)
      d += 7;
    n = (n - d) / 7;
    int yy = (d + 4) / 3 - 1;
    E2 t = mulE(E2{d - 2 * yy, yy}, pw);
    acc.x += t.x;
    acc.y += t.y;
    pw = mulE(pw, base);
  }
  return acc;
}
}  // namespace

void wb_size_fit(const double mn[3], const double mx[3], double center[3], double *sideOut)
{
  double minx = fmin(mn[0], mx[0]), maxx = fmax(mn[0], mx[0]);
  double miny = fmin(mn[1], mx[1]), maxy = fmax(mn[1], mx[1]);
  double minz = fmin(mn[2], mx[2]), maxz = fmax(mn[2], mx[2]);
  center[0] = center[1] = center[2] = 0;
  if (maxz <= minz && maxy <= miny && maxx <= minx)
  {
    *sideOut = 0;
    return;
  }
  int e;
  double side = (maxx + maxy + maxz - minx - miny - minz) / 3;
  side /= frexp(side, &e) * 2;   // divide by the significand in [1,2)
  double x = minx - side, y = miny - side, z = minz - side;
  while (x + side <= maxx || y + side <= maxy || z + side <= maxz)
  {
    side *= 2;
    x = (rint((minx + maxx) / side * 8) - 8) * side / 16;
    y = (rint((miny + maxy) / side * 8) - 8) * side / 16;
    z = (rint((minz + maxz) / side * 8) - 8) * side / 16;
  }
  center[0] = x + side / 2;
  center[1] = y + side / 2;
  center[2] = z + side / 2;
  *sideOut = side;
}

void wb_tile_cube(const double mn[3], const double mx[3], double center[3], double *side)
{
  double b[6];
  for (int i = 0; i < 6; i++)
    b[i] = INFINITY;
  const double *pts[2] = {mn, mx};
  for (const double *p : pts)
  {
    for (int i = 0; i < 4; i++)
    {
      double v = p[0] * kWbQuadrantCosSin[2 * i] + p[1] * kWbQuadrantCosSin[2 * i + 1];
      if (v < b[i])
        b[i] = v;
    }
    if (p[2] < b[4])
      b[4] = p[2];
    if (-p[2] < b[5])
      b[5] = -p[2];
  }
  double left = b[0], bottom = b[1], right = -b[2], top = -b[3], low = b[4], high = -b[5];
  double s = right - left;
  if (top - bottom > s)
    s = top - bottom;
  if (high - low > s)
    s = high - low;
  center[0] = (right + left) / 2;
  center[1] = (top + bottom) / 2;
  center[2] = (high + low) / 2;
  *side = s;
}

void wb_snake_size(double tileSide, double desired, int *idx, double *spacing, int *lo, int *hi)
{
  double best = INFINITY;
  int bi = 0;
  for (int i = 0; i < 12; i++)
  {
    double sp = tileSide / kSquareSides[i];
    double diff = fabs(log(sp / desired));
    if (diff < best)
    {
      best = diff;
      bi = i;
    }
  }
  *idx = bi;
  *spacing = tileSide / kSquareSides[bi];
  *lo = kLoLim[bi];
  *hi = kHiLim[bi];
}

void wb_flowsnake_order(int idx, std::vector<int32_t> &ex, std::vector<int32_t> &ey)
{
  long long count = (long long)kHiLim[idx] - kLoLim[idx] + 1;
  ex.resize(count);
  ey.resize(count);
  for (long long k = 0; k < count; k++)
  {
    E2 e = toEisenstein(curveDigits((int)(kLoLim[idx] + k)));
    ex[k] = (int32_t)e.x;
    ey[k] = (int32_t)e.y;
  }
}

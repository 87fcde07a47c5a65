/* Device-side helpers shared by the kernels.
 *
 * The library is compiled with -fmad=false, so every double expression below
 * rounds exactly like the reference's x86-64 build (no fused multiply-add);
 * the FP32 filters that may use FMA call __fmaf_rn explicitly.
 */
#ifndef WB_DEVICE_CUH
#define WB_DEVICE_CUH
#include <cstdint>
#include <cuda_runtime.h>

#define WB_LEVELS 21          /* Morton levels below the root (3 x 21 = 63 key bits) */
#define WB_RECORDS 537        /* points per block, octree.h:40-42                     */
#define WB_DEG30 0x0aaaaaab
#define WB_DEG45 0x10000000
#define WB_DEG90 0x20000000
#define WB_DEG144 0x33333333
#define WB_DEG180 0x40000000

struct WbDecode
{
  double off[3], scale[3], unit;
};

/* Root cube of the octree: lo = center - side/2 (exact: sizeFit puts it on the
 * side/16 grid) and the cell edge at level 21. */
struct WbRoot
{
  double lo[3];
  double side;
  double cell;   /* side / 2^21 */
};

/* LasHeader::readPoint (las.cpp:808): (offset + scale*X) * unit. */
__device__ __forceinline__ double wb_decode(int32_t q, double off, double scale, double unit)
{
  return (off + scale * (double)q) * unit;
}

/* Index of the level-21 cell that the reference's descent (x >= center at
 * every level, octree.cpp:199-216) puts x in: the largest k with
 * lo + k*cell <= x, clamped to [0, 2^21-1].  Node centres and cell
 * boundaries are exact dyadic doubles, so comparing against them reproduces
 * every >= decision of the descent. */
__device__ __forceinline__ uint32_t wb_cell_index(double x, double lo, double cell)
{
  const int kMax = (1 << WB_LEVELS) - 1;
  // cell = root side / 2^21 and the root side is a power of two, so the
  // product with its reciprocal is the exact quotient (no FP64 division)
  double t = (x - lo) * (1.0 / cell);
  int k;
  if (!(t > 0))
    k = 0;
  else if (t >= (double)kMax)
    k = kMax;
  else
    k = (int)t;
  while (k < kMax && x >= lo + (double)(k + 1) * cell)
    k++;
  while (k > 0 && x < lo + (double)k * cell)
    k--;
  return (uint32_t)k;
}

/* Spreads the low 21 bits of v to every third bit. */
__device__ __forceinline__ uint64_t wb_spread3(uint32_t v)
{
  uint64_t x = v & 0x1fffff;
  x = (x | (x << 32)) & 0x1f00000000ffffULL;
  x = (x | (x << 16)) & 0x1f0000ff0000ffULL;
  x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
  x = (x | (x << 2)) & 0x1249249249249249ULL;
  return x;
}

/* Morton key: per level the octant number z*4 + y*2 + x (octree.cpp:204-207),
 * most significant level first, so ascending keys are depth-first order. */
__device__ __forceinline__ uint64_t wb_morton(uint32_t ix, uint32_t iy, uint32_t iz)
{
  return (wb_spread3(iz) << 2) | (wb_spread3(iy) << 1) | wb_spread3(ix);
}

/* Number of levels (0..21) on which two keys agree from the top. */
__device__ __forceinline__ int wb_common_levels(uint64_t a, uint64_t b)
{
  uint64_t d = a ^ b;
  if (d == 0)
    return WB_LEVELS;
  return (__clzll(d) - 1) / 3;
}

__device__ __forceinline__ void wb_two_sum(double a, double b, double &s, double &e)
{
  s = a + b;
  double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

/* ---- hypot ----
 * dist() and Hyperboloid/Cylinder::in (point.cpp:189-192, shape.cpp:127-135,
 * 214-218) call the C library's hypot.  The glibc that the reference is built
 * against computes it with the corrected square root of C. F. Borges, "An
 * Improved Algorithm for hypot(a,b)" (arXiv:1904.09481, 2019), non-fused
 * form: h = sqrt(x^2+y^2) followed by one Newton-like correction whose terms
 * are arranged to be exact.  That is not correctly rounded (about 0.6% of
 * arguments end one ulp away), so the same steps are used here to give the
 * same doubles.  Arguments are coordinate differences, far from overflow. */
__device__ __forceinline__ double wb_hypot(double a, double b)
{
  double ax = fabs(a), ay = fabs(b);
  if (ay > ax)
  {
    double t = ax;
    ax = ay;
    ay = t;
  }
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

/* ---- atan2i (angle.cpp:117-155) ----
 * Bisection over the tangent table, rotation by the table's sin/cos, then a
 * cubic correction whose sum the reference forms in 64-bit long double and
 * rounds with lrint; here that sum is carried in double-double, which rounds
 * to the same integer unless the sum lies within about 2^-44 of a half. */
__device__ __forceinline__ int wb_atan2i(double y, double x, const double *__restrict__ tanT,
                                         const double *__restrict__ sinT, const double *__restrict__ cosT,
                                         double scaleHi, double scaleLo)
{
  int ret = 0, h;
  double t;
  if (x < 0)
  {
    ret += (y > 0) ? WB_DEG180 : -WB_DEG180;
    y = -y;
    x = -x;
  }
  if (y > x)
  {
    ret += WB_DEG90;
    t = x;
    x = y;
    y = -t;
  }
  if (-y > x)
  {
    ret -= WB_DEG90;
    t = x;
    x = y;
    y = t;
    x = -x;
  }
  t = y / x;
  for (h = WB_DEG45 / 2; h > WB_DEG45 / 1024; h /= 2)
    if (t > tanT[(((ret + WB_DEG45) & 0x1ff00000) >> 20) - 1])
      ret += h;
    else
      ret -= h;
  h = 511 - (((ret + WB_DEG45) & 0x1ff00000) >> 20);
  t = x * cosT[h] - y * sinT[h];
  y = y * cosT[h] + x * sinT[h];
  x = t;
  if (x == 0 && y == 0)
    return 0;
  double q = y / x;
  double dcub = 1.1392738508503886e8 * (q * q * q);
  // P = scale * y (double-double)
  double ph = scaleHi * y;
  double pl = fma(scaleHi, y, -ph) + scaleLo * y;
  // Q = P / x
  double qh = ph / x;
  double rem = fma(-qh, x, ph) + pl;
  double ql = rem / x;
  // V = Q - dcub
  double vh, vl;
  wb_two_sum(qh, -dcub, vh, vl);
  vl += ql;
  double nr = rint(vh);
  double fr = (vh - nr) + vl;
  if (fr > 0.5)
    nr += 1;
  else if (fr < -0.5)
    nr -= 1;
  else if (fr == 0.5 || fr == -0.5)
  {
    double cand = nr + (fr > 0 ? 1 : -1);
    if (fmod(cand, 2.0) == 0)
      nr = cand;
  }
  return ret + (int)nr;
}

/* Cube of a leaf from its key and level, as Octree::cube builds it by
 * halving (octree.cpp:349-358); every value is an exact dyadic double. */
__device__ __forceinline__ void wb_leaf_cube(uint64_t key, int lev, const double *lo, double rootSide, double &cx,
                                             double &cy, double &cz, double &side)
{
  uint32_t ix = 0, iy = 0, iz = 0;
  for (int d = 1; d <= lev; d++)
  {
    int oct = (int)((key >> (63 - 3 * d)) & 7);
    ix = (ix << 1) | (oct & 1);
    iy = (iy << 1) | ((oct >> 1) & 1);
    iz = (iz << 1) | ((oct >> 2) & 1);
  }
  side = ldexp(rootSide, -lev);
  cx = lo[0] + ((double)ix + 0.5) * side;
  cy = lo[1] + ((double)iy + 0.5) * side;
  cz = lo[2] + ((double)iz + 0.5) * side;
}

/* Shape::closestPoint of a cube for a shape whose axis passes through
 * (ax, ay): the coordinate of the nearest face, or ax itself when it lies
 * strictly inside the slab (shape.cpp:137-159, 220-238). */
__device__ __forceinline__ double wb_clamp_toward(double a, double c, double side)
{
  if (fabs(a - c) < side / 2)
    return a;
  return a > c ? c + side / 2 : c - side / 2;
}

/* Direction of (dx, dy) in the reference's angle unit (2^31 per turn) in
 * FP32, for the fast classify filter.  atan on [0,1] is an odd polynomial
 * of degree 11 fitted here by Chebyshev-weighted least squares (maximum
 * error 1.75e-6 rad evaluated in FP32); the octant is restored from the
 * signs and the larger component.  With the fast division and the unit
 * conversion the error stays below 1000 units; callers allow 4096. */
__device__ __forceinline__ float wb_dir_units_f32(float dy, float dx)
{
  float ax = fabsf(dx), ay = fabsf(dy);
  float t = __fdividef(fminf(ax, ay), fmaxf(ax, ay));
  float t2 = t * t;
  float p = -0x1.800344p-7f;
  p = __fmaf_rn(p, t2, 0x1.af4986p-5f);
  p = __fmaf_rn(p, t2, -0x1.dce206p-4f);
  p = __fmaf_rn(p, t2, 0x1.8c5ee6p-3f);
  p = __fmaf_rn(p, t2, -0x1.549b14p-2f);
  p = __fmaf_rn(p, t2, 0x1.fffd04p-1f);
  float th = p * t;
  if (ay > ax)
    th = 1.57079637f - th;
  if (dx < 0)
    th = 3.14159274f - th;
  if (dy < 0)
    th = -th;
  return th * 341782637.79f;   // 2^30 / pi
}

/* Hyperboloid::in (shape.cpp:127-135) for slope > 0, exact double form. */
__device__ __forceinline__ bool wb_hyp_in(double cx, double cy, double cz, double por2, double slope,
                                         double qx, double qy, double qz)
{
  double xyd = wb_hypot(cx - qx, cy - qy);
  double zd = cz - qz;
  if (slope > 0)
    return zd > 0 && zd * zd - (xyd * slope) * (xyd * slope) >= por2;
  return zd < 0 && zd * zd - (xyd * slope) * (xyd * slope) >= por2;
}

#endif

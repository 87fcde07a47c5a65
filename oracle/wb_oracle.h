/* CPU restatement of wolkenbase's classification hot path -- TEST INFRASTRUCTURE.
 *
 * This library is the oracle that the tests, the smoke check and the CPU arm
 * of bench.py compare the CUDA path against.  It is never linked into, called
 * by, or shipped with the product library (libwolkenbase_gb300.so).
 *
 * Pinning: tests/test_oracle_golden.py checks every entry point here against
 * golden vectors written by the reference's own sources compiled here
 * (oracle/_ref/wb_ref, recipe in oracle/Makefile, generator in
 * tests/golden/make_golden.py): atan2i tables and values, least squares,
 * flowsnake addresses, leaf cubes, serial block numbers and storage order,
 * per-tile scan results and per-point classes.
 */
#ifndef WB_ORACLE_H
#define WB_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct
{
  double tile_size;        /* WolkenCanvas::tileSize, default 1 m        */
  double max_slope;        /* maxSlope (scan.cpp:29), default 1          */
  double thickness;        /* thickness, default 0                       */
  double min_hyp_size;     /* minHyperboloidSize, default 0.1 m          */
} wbo_params;

typedef struct
{
  /* inputs */
  const int32_t *xyz;      /* n x 3 LAS integers                        */
  uint64_t n;
  double scale[3], offset[3], unit;
  double minc[3], maxc[3]; /* header corners in file units              */
  int phases;              /* 1 build, 2 +scan/postscan, 3 +classify    */
  int canonical_order;     /* 0: serial storage order (as the reference's
                              single-threaded driver); 1: each block's
                              points ordered by input index             */
  int threads;             /* worker threads for scan/classify (>=1)    */
  /* outputs (caller-allocated, n entries unless noted; may be NULL) */
  int64_t *block;          /* serial block number, -1 if overwritten dup */
  int32_t *block_pos;      /* position within the block's storage        */
  int64_t *leaf;           /* leaf index in depth-first (sub[0..7]) order */
  uint8_t *cls;            /* class written by classify (0 if untouched) */
  /* summary outputs */
  uint64_t n_blocks, n_leaves, n_tiles;
  double root_center[3], root_side;
  double snake_center[3], snake_side, spacing;
  int snake_index;         /* which Gosper island size was chosen        */
  double t_build, t_scan, t_postscan, t_classify;  /* seconds */
  /* Sampled run (n_sample > 0, phases >= 2): only these tiles (positions in
     flowsnake order, 0-based) are post-scanned and classified; the tiles
     their postscan walks are scanned on demand.  cls is written only for the
     stored points whose last containing tile in flowsnake order is sampled,
     so every written byte is final. */
  const int64_t *sample_tiles;
  uint64_t n_sample;
  uint64_t n_scanned;      /* tiles scanned (sampled run: the sample plus what postscan needed) */
  uint64_t n_sample_points;   /* points in the sampled tiles' cylinders (classified, overlaps counted) */
  double *margin;          /* full run, optional (n): the deciding tile's largest direction gap of
                              each point at the end of its loop, in degrees minus 144 (216 with
                              fewer than two directions; NaN for points no tile holds) */
} wbo_run_io;

/* Whole pipeline; returns 0 on success. */
int wbo_run(wbo_run_io *io, const wbo_params *p);

/* After wbo_run: leaf table in depth-first order (center xyz, side, count). */
int wbo_leaves(double *center_side /* n_leaves x 4 */, int64_t *count /* n_leaves */);

/* After wbo_run with phases>=2: tiles in flowsnake order. */
typedef struct
{
  int32_t ex, ey, n_points, n_ground, tree_flags, pad;
  double density, h_scan, h_final, height;
} wbo_tile;
int wbo_tiles(wbo_tile *out /* n_tiles */);

/* After wbo_run: another sampled run (see sample_tiles above) over the same
 * octree, from a fresh tile table; cls has one entry per input point. */
int wbo_sample(const int64_t *tiles, uint64_t count, int threads, uint8_t *cls, double *t_scan, double *t_classify,
               uint64_t *n_scanned, uint64_t *n_points);

/* After wbo_run(keep): OctStore::pointsIn of a Cylinder (kind 1: v[0], v[1],
 * radius r) or a Hyperboloid (kind 2: vertex v, r, slope s) as input point
 * indices (sorted: by height, ties in unsorted order), and Octree::findBlocks
 * as depth-first leaf indices; each returns the full count (at most capacity
 * entries written), -1 on error. */
int64_t wbo_points_in(int kind, const double *v, double r, double s, int sorted, uint32_t *out, uint64_t capacity);
int64_t wbo_find_blocks(int kind, const double *v, double r, double s, int64_t *out, uint64_t capacity);

/* Tiles of the flowsnake island Flowsnake::setSize picks for a cloud with
 * these header corners (file units) and tile size. */
int64_t wbo_snake_tiles(const double *minc, const double *maxc, double unit, double tile_size);

/* Frees the state kept by wbo_run. */
void wbo_reset(void);

/* Primitives restated from the reference, for golden-vector tests. */
void wbo_fill_tables(double *tan511, double *sin512, double *cos512);
void wbo_set_tables(const double *tan511, const double *sin512, const double *cos512);
int32_t wbo_atan2i(double y, double x);
void wbo_atan2i_many(const double *yx, uint64_t n, int32_t *out);
void wbo_quadrant_trig(double *cos_sin8);
double wbo_pairwisesum(const double *a, unsigned n);
void wbo_hypot_many(const double *ab, uint64_t n, double *out);
void wbo_lsq_plane(const double *xyz, uint64_t rows, double *out3);
int wbo_hyperboloid_in(const double *vertex, double r, double s, const double *pnt);
int wbo_cylinder_in(const double *center_xy, double r, const double *pnt);
void wbo_size_fit(const double *minc, const double *maxc, double *center3, double *side);
void wbo_flowsnake(int size_index, int32_t *exy /* 2*(hi-lo+1) */);
int wbo_flowsnake_limits(int size_index, int32_t *lo, int32_t *hi);

#ifdef __cplusplus
}
#endif
#endif

/* wolkenbase_gb300 -- GPU (sm_103a) replacement for wolkenbase's classification
 * hot path behind a plain C ABI.
 *
 * The reference runs this path in-process through C++ globals:
 *   Octree octRoot / OctStore octStore   (octree.h:55-212, octree.cpp:37-38)
 *   Flowsnake snake, harray<Tile> tiles  (threads.cpp:69, tile.cpp:27)
 *   scanCylinder / postscanCylinder      (scan.h:27-28)
 *   classifyCylinder                     (classify.h:24)
 * driven phase by phase by WolkenThread (threads.cpp:446-695).  Here one
 * context owns the device-resident octree, point store and tile table for one
 * cloud; each call below replaces one of those phases for the whole cloud.
 *
 * Conventions: every function returns 0 on success or a negative WB_E* code;
 * wb_last_error() describes the last failure.  No exception crosses the ABI.
 * The caller owns every host array; the context owns all device memory.  A
 * context is not thread-safe: use one per host thread.  Host arrays may be
 * pageable or pinned; pinned buffers make the copies asynchronous.
 */
#ifndef WOLKENBASE_GB300_H
#define WOLKENBASE_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WB_OK 0
#define WB_EINVAL -1      /* bad argument                                    */
#define WB_ENOMEM -2      /* device allocation failed or HBM budget exceeded */
#define WB_ECUDA -3       /* a CUDA call failed                              */
#define WB_EDEPTH -4      /* a leaf would lie deeper than 21 levels          */
#define WB_ESTATE -5      /* call out of order (e.g. classify before build)  */
#define WB_ETIMEDOUT -6   /* a bounded device-side wait gave up              */
#define WB_ENOTFOUND -7   /* no such job / entry                             */
#define WB_EBUSY -8       /* job already running or finished (wb_cancel)     */
#define WB_ECANCELED -9   /* job was cancelled before it ran                 */
#define WB_EIO -10        /* a file could not be written                    */

/* Classify kernel shapes: one warp per group of up to 32 points of a grid
 * column (0-2) or one warp per point (3-7); warps per block / resident blocks
 * per SM (register cap): 0 = groups 4/5 (default), 1 = groups 8/3,
 * 2 = groups 8/2, 3 = 8/3, 4 = 4/6, 5 = 4/8, 6 = 8/4, 7 = 2/12. */
#define WB_N_SHAPES 8

typedef struct wb_ctx wb_ctx;

/* Classification settings; defaults as MainWindow::readSettings
 * (mainwindow.cpp:407-410) and scan.cpp:29. */
typedef struct
{
  double tile_size;     /* WolkenCanvas::tileSize, 1 m        */
  double max_slope;     /* maxSlope, 1                        */
  double thickness;     /* thickness, 0 m                     */
  double min_hyp_size;  /* minHyperboloidSize, 0.1 m          */
} wb_params;

/* One LAS point block as LasHeader::readPoint sees it (las.cpp:735-820).
 * records[i*stride + 0..11] hold the little-endian int32 X, Y, Z of point i
 * (true for every LAS point format); stride is the point record length
 * (12 for packed XYZ, 28 for format 1).  Coordinates decode as
 * (offset + scale*X) * unit, exactly las.cpp:808.  minc/maxc are the header's
 * min/max corner in file units (LasHeader::minCorner/maxCorner, las.cpp:704-712),
 * which size the octree root and the tile grid (wolkencanvas.cpp:497-520). */
typedef struct
{
  const void *records;
  uint64_t n;
  uint32_t stride;
  uint32_t device_resident;   /* 1: records is a device pointer      */
  double scale[3], offset[3], unit;
  double minc[3], maxc[3];
} wb_cloud;

typedef struct
{
  uint64_t n_points;        /* input records                                    */
  uint64_t n_distinct;      /* after exact-xyz de-duplication (octree.cpp:620-644) */
  uint64_t n_leaves;        /* leaf blocks (OctStore::getNumBlocks, octree.h:168) */
  uint32_t max_depth;       /* deepest leaf level below the root                */
  uint32_t pad;
  double root_center[3], root_side;    /* Octree::sizeFit (octree.cpp:268-310)  */
  double tile_center[3], tile_side;    /* cube handed to Flowsnake::setSize     */
  double spacing;                       /* Flowsnake::getSpacing                 */
  uint64_t n_tiles;                     /* Gosper island size (hiLim-loLim+1)    */
  int32_t tile_lo, tile_hi;             /* flowsnake counter range               */
} wb_octree_stats;

/* Per-tile results of scan + postscan (Tile, tile.h:27-35), flowsnake order. */
typedef struct
{
  int32_t ex, ey;            /* Eisenstein tile address                    */
  int32_t n_points, n_ground;
  int32_t tree_flags, pad;
  double density, h_scan, hyperboloid_size, height;
} wb_tile;

/* Replaces octStore.open + startThreads (wolkenbase.cpp:75-76, threads.cpp:91).
 * device: CUDA ordinal.  hbm_budget: bytes this context may allocate (0 = no
 * limit).  Returns NULL on failure (see wb_last_error(NULL)). */
wb_ctx *wb_open(int device, size_t hbm_budget);
void wb_close(wb_ctx *ctx);
const char *wb_last_error(const wb_ctx *ctx);
/* Work is issued on this stream (a cudaStream_t); NULL = the context's own. */
int wb_set_stream(wb_ctx *ctx, void *cuda_stream);
int wb_synchronize(wb_ctx *ctx);

/* Paging for clouds above the HBM budget (the reference pages octree blocks
 * to store.oct through an LRU cache under lowRam back-pressure:
 * octree.cpp:427-559, 1017-1147; threads.cpp:227-228).  Here buffers that do
 * not fit the context's HBM budget are placed in pinned host memory -- on
 * GB300 the Grace LPDDR5X behind NVLink-C2C -- and the kernels use them in
 * place; a cloud whose working set is above the budget puts its sequential
 * scratch buffers (sort ping-pong, record upload, tile lists) there first so
 * that HBM keeps what the classify reads at random.  host_budget: bytes of
 * host memory the context may pin (0 = off, the default: over-budget
 * allocations fail with WB_ENOMEM).  Needs a device that uses host memory in
 * place with native atomics (WB_EINVAL otherwise). */
int wb_set_paging(wb_ctx *ctx, size_t host_budget);
/* Host bytes held now and at most, and device bytes held now. */
int wb_paging_stats(wb_ctx *ctx, uint64_t *host_bytes, uint64_t *host_peak, uint64_t *device_bytes);

/* Octree::sizeFit + OctStore::put for every record + OctStore::split
 * (octree.cpp:268-347, 620-662, 849-876, 1295-1338).  Leaf cubes and the
 * point->leaf map equal the reference's; leaves are numbered in depth-first
 * sub[0..7] order (the order Octree::findBlocks visits them).  Asynchronous
 * on the context's stream. */
int wb_octree_build(wb_ctx *ctx, const wb_cloud *cloud);
int wb_octree_info(wb_ctx *ctx, wb_octree_stats *out);

/* Leaf table: center xyz + side (4 doubles per leaf), first store slot and
 * point count per leaf (Octree::cube + OctBuffer::countPoints). */
int wb_octree_leaves(wb_ctx *ctx, double *center_side, uint32_t *first, uint32_t *count);

/* Octree::findBlock for every input record: leaf index (same numbering). */
int wb_octree_point_leaf(wb_ctx *ctx, uint32_t *leaf_of_point);

/* The point store: input index of each distinct point in store order (leaf
 * by leaf; inside a leaf by input index, the survivor of duplicates being
 * the last one read, as OctBuffer::put keeps it). */
int wb_octree_store_order(wb_ctx *ctx, uint32_t *input_index);

/* Octree::findBlock for arbitrary positions (m xyz triples, doubles):
 * leaf index, or -1 where findBlock would return -1. */
int wb_octree_find_block(wb_ctx *ctx, const double *xyz, uint64_t m, int64_t *leaf);

/* wb_octree_find_block without any device allocation (no counterpart in the
 * reference).  Some callers of this library cannot afford cudaMalloc/cudaFree
 * on the query path: cudaFree waits for the whole device, so a serving loop
 * that answers point lookups between classification jobs would stall every
 * job in flight, and a process running close to its HBM budget (many clouds
 * resident) may have no room left for even a small staging allocation.  This
 * entry point stages positions and results in a file-scope device array of
 * WB_FIND_BLOCK_STATIC_MAX entries that every GPU loading the library keeps
 * until the process exits (about 2 MB per GPU).  Its first call on a device
 * looks the array's address up (cudaGetSymbolAddress); make that first call
 * before any stream capture.  m above WB_FIND_BLOCK_STATIC_MAX is rejected
 * with WB_EINVAL.  All calls share the one array: calls that overlap on the
 * GPU (two host threads, or two contexts on one device) race and must be
 * serialised by the caller.  Every result slot is written by each call, so
 * nothing left over from an earlier call is read.  Like every context on
 * that device, the looked-up address does not survive cudaDeviceReset of the
 * device: a process that resets a device must not use this library on it
 * again.  Synchronous. */
#define WB_FIND_BLOCK_STATIC_MAX 65536
int wb_octree_find_block_static(wb_ctx *ctx, const double *xyz, uint64_t m, int64_t *leaf);

/* A shape of the neighbourhood queries, as the reference constructs them:
 * WB_SHAPE_CYLINDER    Cylinder(xy c, double r) (shape.cpp:207-218):
 *                      v[0], v[1] = c, r = radius (any height)
 * WB_SHAPE_HYPERBOLOID Hyperboloid(xyz v, double r, double s) (shape.cpp:
 *                      119-135): vertex v, radius of curvature r, slope s
 *                      (s > 0 opens downward, as classifyCylinder uses it) */
#define WB_SHAPE_CYLINDER 1
#define WB_SHAPE_HYPERBOLOID 2
typedef struct
{
  int kind;
  int pad;
  double v[3];
  double r, s;
} wb_shape;

/* Octree::findBlocks (octree.cpp:234-251): the leaves whose cube the shape
 * intersects, depth-first (the leaf numbering).  *count receives how many;
 * WB_EINVAL when that exceeds capacity (nothing written).  Synchronous. */
int wb_find_blocks(wb_ctx *ctx, const wb_shape *shape, int64_t *leaves, uint64_t capacity, uint64_t *count);

/* OctStore::pointsIn (octree.cpp:1214-1242): the stored points the shape
 * holds -- every point of a block whose cube's eight corners are inside,
 * the points inside for the other blocks findBlocks returns -- as input
 * record indices (the surviving record of a duplicated location), blocks
 * depth-first and store order inside a block; sorted != 0 orders them by
 * height (ties keep that order; the reference's std::sort leaves them in no
 * particular order).  *count receives how many; WB_EINVAL when that exceeds
 * capacity (nothing written).  Synchronous. */
int wb_points_in(wb_ctx *ctx, const wb_shape *shape, int sorted, uint32_t *records, uint64_t capacity,
                 uint64_t *count);

/* scanCylinder over every tile then postscanCylinder over every tile
 * (scan.cpp:31-179), in flowsnake order. */
int wb_scan_tiles(wb_ctx *ctx, const wb_params *params);
int wb_tiles(wb_ctx *ctx, wb_tile *out, uint64_t capacity, uint64_t *count);

/* classifyCylinder over every tile (classify.cpp:96-173).  cls is per input
 * record: on entry the caller's current class byte (the LAS classification,
 * 0 for a fresh cloud); on return every point that lies in a tile cylinder
 * holds 1 (not ground) or 2 (ground), written by the last tile in flowsnake
 * order that contains it; other bytes are left unchanged.  cls may be a host
 * or (cls_on_device=1) a device pointer. */
int wb_classify(wb_ctx *ctx, const wb_params *params, uint8_t *cls, int cls_on_device);

/* wb_classify plus each point's decision margin (the margin_out of the
 * classify entry point): margin[i] (per input record, on the side of cls)
 * is, in degrees, the largest circular gap between the directions of the
 * point's hyperboloid neighbours minus 144 (surround, classify.cpp:67-94):
 * negative for class 1, positive for class 2, 216 when fewer than two
 * directions exist, NaN for a record no tile cylinder holds.  A point proven
 * surrounded before all its neighbours were seen reports the gap at that
 * moment (the full set's gap is no larger, so its true margin is at least as
 * far from zero).  Gaps decided by the FP32 filter carry its direction error,
 * below 3.5e-4 degrees; ambiguous points are re-run with exact directions.
 * margin may be NULL (then this is wb_classify). */
int wb_classify_ex(wb_ctx *ctx, const wb_params *params, uint8_t *cls, int cls_on_device, float *margin);

/* Build + scan + postscan + classify in one call. */
int wb_classify_cloud(wb_ctx *ctx, const wb_cloud *cloud, const wb_params *params, uint8_t *cls);

/* Settings of the classify kernel (no reference counterpart; they change
 * speed, never labels): the kernel shape (see WB_N_SHAPES), the points a
 * warp takes per visit to the work counter, and the points per column of
 * the neighbour grid (applies from the next wb_octree_build).  In
 * wb_set_tuning, a negative shape or a zero chunk/grid_points keeps the
 * current value.  wb_autotune times the candidates on the scanned cloud,
 * keeps the fastest, and rebuilds the grid with the chosen density. */
typedef struct
{
  int shape;
  int chunk;
  double grid_points;
} wb_tuning;
int wb_set_tuning(wb_ctx *ctx, const wb_tuning *t);

/* Precision mode (no reference counterpart).  WB_PRECISION_EXACT (default)
 * reproduces the reference bit for bit: FP32 work is only a filter, and
 * every decision inside its error band is re-run in FP64.  WB_PRECISION_FP32
 * runs neighbour distances and the tile fit sums in FP32 in a tile-local
 * frame (Kahan-compensated sums, FP64 3x3 solve) and lets FP32 decisions
 * stand; labels can then differ from the reference for points whose
 * decision margin is within FP32 rounding.  Applies from the next
 * wb_scan_tiles / wb_classify.  Clouds whose record differences do not fit
 * FP32 exactly always run exact. */
#define WB_PRECISION_EXACT 0
#define WB_PRECISION_FP32 1
int wb_set_precision(wb_ctx *ctx, int mode);

/* The least-squares plane of every tile from the last wb_scan_tiles, in
 * flowsnake order: 3 doubles per tile (a, b, c of z = a*x + b*y + c, x and y
 * measured from the tile centre); NaN where the fit is singular.  With
 * WB_PRECISION_FP32 this is the FP32-sum fit. */
int wb_tile_planes(wb_ctx *ctx, double *abc, uint64_t capacity);

/* The per-point fit residuals of every tile (no reference counterpart: the
 * precision report).  r = z - (a*x + b*y + c) over the tile's points, x and y
 * from the tile centre, under the planes of the last wb_scan_tiles and under
 * abc_ref (3 doubles per tile, e.g. wb_tile_planes of an exact scan):
 * max_diff[k] = max |r - r_ref|, max_ref[k] = max |r_ref| (NaN where either
 * plane is singular).  Host arrays of the tile count.  Synchronous. */
int wb_tile_residuals(wb_ctx *ctx, const double *abc_ref, double *max_diff, double *max_ref);
int wb_get_tuning(wb_ctx *ctx, wb_tuning *t);
int wb_autotune(wb_ctx *ctx, const wb_params *params);

/* Timing of the last pipeline run, per stage, from CUDA events on the
 * context's stream (milliseconds).  names/ms arrays of capacity entries;
 * returns the number of stages via *count. */
int wb_stage_times(wb_ctx *ctx, const char **names, float *ms, uint32_t capacity, uint32_t *count);

/* Enables or disables the per-stage events (off by default). */
int wb_profile(wb_ctx *ctx, int enable);

/* Kernels this context has launched since wb_open (no reference counterpart:
 * accounting for timed regions). */
int wb_launch_count(wb_ctx *ctx, uint64_t *count);

/* Self-checks of the device arithmetic (no reference counterpart: they let a
 * caller verify the GPU's integer directions and distances against its own
 * host): atan2i (angle.cpp:117-155) of m (y,x) pairs; hypot as the
 * reference's libm computes it; Hyperboloid::in (shape.cpp:127-135) of m
 * points for vertex v, curvature radius r and slope s.  Synchronous. */
int wb_check_atan2i(const double *yx, uint64_t m, int32_t *out);
int wb_check_hypot(const double *ab, uint64_t m, double *out);
/* The FP32 direction of the classify filter for m record differences
 * (dx, dy) at scales sx, sy, in the reference's angle unit (2^31 per turn,
 * masked to 31 bits like atan2i's result); its error against atan2i bounds
 * the filter's margin. */
int wb_check_dir_f32(const int32_t *dxy, double sx, double sy, uint64_t m, uint32_t *out);
int wb_check_hyperboloid(const double *v, double r, double s, const double *xyz, uint64_t m, uint8_t *out);

/* ---- The steps either side of the path ---- */

/* OctStore::countClasses over every block (octree.cpp:664-671, 878-881;
 * threads.cpp:425-444): totals[c] (256 entries) = stored (distinct) points
 * whose class byte after the last wb_classify is c. */
int wb_class_totals(wb_ctx *ctx, uint64_t *totals);

/* OctBuffer::put's overwrite of an identical point (octree.cpp:620-662):
 * *n_dup = records a later identical point replaced; with dup_of (n entries,
 * may be NULL), the record whose point the store kept, for every record
 * (itself when it survived). */
int wb_duplicates(wb_ctx *ctx, uint64_t *n_dup, uint32_t *dup_of);

/* The class field LasHeader::writePoint writes (las.cpp:853-862), in place
 * in n LAS point records of point_format 0-10: formats 0-5 keep the three
 * flag bits above the 5-bit class, 6-10 take the whole byte.  cls NULL takes
 * the class bytes of the last wb_classify (n must be its record count).
 * records (and cls, when given) are device pointers if on_device. */
int wb_las_write_classes(wb_ctx *ctx, void *records, uint64_t n, uint32_t stride, int point_format, int on_device,
                         const uint8_t *cls);

/* CloudOutput::writeFiles's grouping of the points by class
 * (cloudoutput.cpp:187-231) on the device: out receives the n records
 * grouped by class byte (class ascending, input order within a class);
 * offsets (257 entries) bound each class's records.  The files themselves
 * are the caller's.  records and out are device pointers if on_device. */
int wb_las_split_by_class(wb_ctx *ctx, const void *records, uint64_t n, uint32_t stride, int point_format,
                          int on_device, void *out, uint64_t *offsets);

/* OctStore::hiLoPointsIn and countPointsIn (octree.cpp:1244-1293) for every
 * pixel of a w x h view, each pixel a Column (shape.cpp:245-254) of the given
 * side centred at (x0 + i*side, y0 + j*side), as WolkenCanvas::pixelColorRead
 * (wolkencanvas.cpp:91-106) asks them one at a time.  count (w*h, may be
 * NULL): stored points in the column; lo/hi (w*h doubles each, may be NULL):
 * their lowest and highest elevation, INFINITY/-INFINITY when empty.
 * Pixel p = j*w + i. */
int wb_preview(wb_ctx *ctx, double x0, double y0, double side, int w, int h, uint64_t *count, double *lo, double *hi);

/* ---- LAS records: full decode and the class-split writer ---- */

/* Record length of LAS point formats 0-10 (las.cpp:38); 0 for others. */
int wb_las_point_length(int point_format);

/* The fields of a LasPoint (las.h:53-78) as LasHeader::readPoint fills them
 * (las.cpp:735-820), one array per field, indexed by record.  Any pointer
 * may be NULL (field not wanted).  Fields a format lacks read as LasPoint's
 * defaults (las.cpp:121-132): 0.  scan_angle is in 2^31 units per turn
 * (degtobin, angle.cpp:229-243). */
typedef struct
{
  double *x, *y, *z;               /* (offset + scale*X) * unit, las.cpp:808 */
  uint16_t *intensity, *return_num, *n_returns;
  uint8_t *scan_direction, *edge_line;
  uint16_t *classification, *class_flags, *scanner_channel, *user_data;
  int32_t *scan_angle;
  uint16_t *point_source;
  double *gps_time;
  uint16_t *red, *green, *blue, *nir;
} wb_las_points;

/* readPoint for every record of cloud (formats 0-10; stride >= the format's
 * record length).  The arrays are device pointers if cloud->device_resident,
 * else host pointers. */
int wb_las_decode(wb_ctx *ctx, const wb_cloud *cloud, int point_format, const wb_las_points *out);

/* What CloudOutput is told before openFiles (wolkencanvas.cpp:614-622,
 * cloudoutput.h). */
typedef struct
{
  int32_t point_format;        /* CloudOutput::pointFormat (wb_las_join_point_format)  */
  int32_t separate_classes;    /* one set of files per class (SI_EXTRACT)             */
  int32_t n_input_files;       /* > 1: system identifier MERGE                         */
  int32_t creation_day;        /* day of year (1-366) and year written in the headers; */
  int32_t creation_year;       /* 0 = today (UTC), as LasHeader::openWrite does        */
  int32_t pad;
  uint64_t points_per_file;    /* CloudOutput::pointsPerFile; 0 = one file per set     */
  double unit;                 /* CloudOutput::unit, metres per file unit              */
  double min_cor[3], max_cor[3];   /* CloudOutput::minCor/maxCor, metres                */
  double scale[3];             /* CloudOutput::scale (wb_las_combine_scales), metres   */
  const char *software;        /* header software name; NULL = "Wolkenbase 0.1.2~alpha" */
} wb_las_output;

/* One output file: its place in the set, its records in the output buffer
 * and the header figures LasHeader accumulates while writing (las.cpp:636-673,
 * 822-903). */
typedef struct
{
  int32_t class_id;            /* class of the set; 0 when classes are not separated */
  int32_t index;               /* file number within its set                          */
  int32_t name_digits;         /* digits of that number in the file name              */
  int32_t point_format;
  uint64_t first;              /* first record of the file in the output buffer       */
  uint64_t n_points[16];       /* [0] records, [r] records of return number r         */
  double scale[3], offset[3];  /* LasHeader::setScale, file units                     */
  double min[3], max[3];       /* of the written coordinates, file units (+-INFINITY if empty) */
} wb_las_file;

/* joinPointFormat (las.cpp:103-118): the smallest format whose features
 * hold every input format's. */
int wb_las_join_point_format(const int *formats, int n);

/* combineScales (las.cpp:906-944): per axis, the scale that fits every input
 * file's scale and offset (manygcd, manygcd.cpp:44-74).  scales and offsets
 * are n x 3 (metres: LasHeader::getScale/getOffset); out receives 3. */
int wb_las_combine_scales(const double *scales, const double *offsets, int n, double *out);

/* CloudOutput::openFiles + writeFiles (cloudoutput.cpp:116-231) on the
 * device: every stored point of the classified cloud is read from its record
 * (the surviving record of a duplicated location), given its class byte and
 * written with LasHeader::writePoint (las.cpp:822-904) into the file of its
 * class, files balanced by points_per_file over the octree's blocks.
 * cls: class byte per record (NULL = those of the last wb_classify), on the
 * side of the records.  out receives the files' records back to back
 * (n_distinct x wb_las_point_length(opt->point_format) bytes; device pointer
 * if out_on_device).  files (max_files entries) receive each file;
 * *n_files their count, also when max_files is too small (WB_EINVAL). */
int wb_las_write_output(wb_ctx *ctx, const wb_cloud *cloud, int in_format, const uint8_t *cls,
                        const wb_las_output *opt, void *out, int out_on_device, wb_las_file *files, int max_files,
                        int *n_files);

/* LasHeader::writeHeader (las.cpp:540-595) of one output file: 375 bytes of
 * a LAS 1.4 header.  Fields the reference leaves unset (source id, global
 * encoding, GUID, start of waveform data) are written as 0. */
int wb_las_header_bytes(const wb_las_output *opt, const wb_las_file *file, uint8_t *header);

/* The name CloudOutput::openFiles gives a file (cloudoutput.cpp:146-185):
 * base-class[-NN].las, or base[-NN].las when classes are not separated. */
int wb_las_file_name(const wb_las_output *opt, const wb_las_file *file, const char *base, char *buf, size_t cap);

/* wb_las_write_output, then every file written to disk under its name
 * (header + records), as writeFiles + closeFiles (cloudoutput.cpp:187-245). */
int wb_las_write_files(wb_ctx *ctx, const wb_cloud *cloud, int in_format, const uint8_t *cls,
                       const wb_las_output *opt, const char *base, wb_las_file *files, int max_files, int *n_files);

/* ---- Serving and batching ----
 *
 * No reference counterpart as an API: the reference runs one cloud at a time
 * through WolkenCanvas::startProcess and the TH_* phases of WolkenThread
 * (wolkencanvas.cpp:469-532, threads.cpp:547-660).  A server takes
 * tile-classify jobs as they arrive and runs each through the same path as
 * wb_classify_cloud (same results, bit for bit): up to prep_slots jobs are
 * built and scanned at once on their own streams, each job's octree and point
 * buffers stay on the device until its class bytes are out, and jobs whose
 * scan has finished are classified together by one fused, graph-captured
 * launch over all their points.  A job is admitted only while the device
 * memory all admitted jobs hold, plus its own estimate, stays within
 * hbm_budget; jobs start in submission order. */
typedef struct wb_server wb_server;

#define WB_FLUSH_EAGER 0   /* classify whatever has been scanned (serving)            */
#define WB_FLUSH_FULL 1    /* wait until every admitted job is scanned (batching)     */

typedef struct
{
  int device;
  int prep_slots;        /* jobs built and scanned concurrently; 0 = 4              */
  uint64_t hbm_budget;   /* bytes all resident jobs may hold; 0 = 80% of free memory */
  int flush;             /* WB_FLUSH_EAGER or WB_FLUSH_FULL                         */
  int max_batch;         /* most jobs in one fused classify launch; 0 = 512 (max)   */
  int shape;             /* fused fast-pass kernel shape, 0..WB_N_SHAPES-1 (below)  */
  int chunk;             /* groups (or points) a warp takes per visit to the work counter; 0 = 1 */
  double grid_points;    /* points per column of the neighbour grid; 0 = 64         */
  int autotune;          /* 1: on the first batch, time column densities, kernel
                            shapes and chunks on a sample and keep the fastest     */
  int pad;
  uint64_t host_budget;  /* > 0: a job whose estimate is above hbm_budget runs alone
                            with paging (wb_set_paging) up to this many host bytes,
                            instead of failing with WB_ENOMEM                      */
} wb_server_config;

typedef struct
{
  wb_cloud cloud;        /* records stay valid and unchanged until the job ends     */
  wb_params params;
  uint8_t *cls;          /* n class bytes, host memory, as for wb_classify          */
  uint64_t tag;          /* caller's value, returned in wb_job_status               */
} wb_job;

#define WB_JOB_QUEUED 0
#define WB_JOB_PREP 1       /* building the octree and scanning the tiles */
#define WB_JOB_READY 2      /* scanned, waiting for a fused classify      */
#define WB_JOB_CLASSIFY 3
#define WB_JOB_DONE 4
#define WB_JOB_FAILED 5
#define WB_JOB_CANCELLED 6

typedef struct
{
  int state;                 /* WB_JOB_*                                              */
  int rc;                    /* 0, or the WB_E* code of a failed or cancelled job     */
  uint64_t tag;
  uint64_t n_points, n_ground, n_ambiguous;
  uint64_t reserved_bytes;   /* device memory the job was admitted against            */
  double t_submit, t_admit, t_ready, t_done;   /* seconds on the server's clock      */
  int batch_jobs;            /* jobs in the fused classify launch it ran in           */
  int pad;
} wb_job_status;

typedef struct
{
  uint64_t submitted, completed, failed, cancelled;
  uint64_t points;           /* input records of completed jobs                       */
  uint64_t fused_launches, fused_jobs;
  uint64_t held_bytes, peak_bytes, budget;
  uint64_t kernel_launches;  /* kernels the server's contexts and graphs launched     */
  int contexts, queued, running, pad;
  double now;                /* the server's clock                                    */
  int tuned;                 /* 1 once the autotuner has run                          */
  int shape, chunk, pad2;    /* fast-pass shape and chunk in use                      */
  double grid_points;        /* column density in use                                 */
  double tune_ms;            /* time the autotuner took                               */
} wb_server_stats;

wb_server *wb_server_open(const wb_server_config *cfg);   /* NULL on error: wb_last_error(NULL) */
void wb_server_close(wb_server *s);                       /* cancels queued jobs, waits for running ones */
const char *wb_server_error(const wb_server *s);
/* Returns the job id (>= 0) or a WB_E* code. */
int64_t wb_submit(wb_server *s, const wb_job *job);
int wb_poll(wb_server *s, int64_t id, wb_job_status *st);
/* Waits until the job is done, failed or cancelled, or timeout_s passes
 * (WB_ETIMEDOUT); timeout_s < 0 waits without limit. */
int wb_wait(wb_server *s, int64_t id, double timeout_s, wb_job_status *st);
/* Cancels a queued job; WB_EBUSY once it has been admitted. */
int wb_cancel(wb_server *s, int64_t id);
/* Forgets a finished job's status. */
int wb_release(wb_server *s, int64_t id);
int wb_server_stats_get(wb_server *s, wb_server_stats *out);
/* Runs k jobs (the C++ adapter's TH_SCAN/TH_SPLIT over many clouds) and waits
 * for all; rcs[i] receives each job's code.  Returns 0 if all succeeded. */
int wb_classify_batch(wb_server *s, const wb_job *jobs, int k, int *rcs);

#ifdef __cplusplus
}
#endif
#endif

/*
 * rtr.h — C ABI of the GB300 (sm_103a) model-to-scene registration hot path.
 *
 * This is the drop-in boundary for the registration chain of ICCD/RealTime_Robot
 * (RealTimeRobot/RealTimeRobot.cpp:27-121 driving key_point.h, matching.h,
 * model_point.h, scan_point.h and function.h).  The reference reaches the GPU
 * through exactly one C entry point, ComputeTDFWithCuda (kernel.cu:34-106,
 * declared at key_point.h:35-36); it is kept below with its exact signature.
 * Everything else the reference does through PCL on the CPU is offered here as
 * rtr_* entry points that the C++ entry points (ModelPoint, ScanPoint,
 * KeyPoint, get_Distance, Ransac, keyPointICP, match_by_*) call.
 *
 * Conventions (all rtr_* calls):
 *   - Plain pointers and sizes only.  "d_" pointers are device pointers, "h_"
 *     pointers are host pointers.  The caller owns every input and output
 *     buffer; the context owns scratch memory.
 *   - Point clouds are arrays of 16-byte points {x, y, z, pad} (float), the
 *     memory layout of pcl::PointXYZ.  The pad lane is ignored on input.
 *   - Poses are row-major 4x4 doubles mapping source coordinates into target
 *     coordinates: q = R p + t.
 *   - Work is enqueued on the given stream (0 = legacy default stream) and the
 *     call returns without synchronising unless its comment says otherwise.
 *   - Every call returns an rtr_status; no C++ exception crosses the ABI.  The
 *     text of the last failure is available from rtr_last_error().
 *   - A context is used by one host thread at a time.
 */
#ifndef RTR_H_
#define RTR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__CUDA_RUNTIME_H__) || defined(__CUDACC__)
typedef cudaStream_t rtr_stream_t;
#else
typedef struct CUstream_st* rtr_stream_t;
#endif

typedef enum rtr_status {
  RTR_OK = 0,
  RTR_ERR_INVALID_ARG = 1,  /* bad pointer, size or parameter                 */
  RTR_ERR_OOM = 2,          /* device allocation failed                       */
  RTR_ERR_TIMEOUT = 3,      /* a bounded device-side wait ran out             */
  RTR_ERR_NOT_FOUND = 4,    /* no model instance / correspondence was found   */
  RTR_ERR_CUDA = 5,         /* a CUDA runtime call failed                     */
  RTR_ERR_CAPACITY = 6,     /* scratch too small while a stream is captured   */
  RTR_ERR_NO_DEVICE = 7     /* no usable sm_103a device                       */
} rtr_status;

typedef struct rtr_context rtr_context;
typedef struct rtr_mlp rtr_mlp;   /* learned keypoint credibility (below) */

/* ---- library / context ------------------------------------------------- */

const char* rtr_status_string(int status);
/* Text of the last failure recorded on this host thread ("" if none). */
const char* rtr_last_error(void);
/* Library version, e.g. "0.1.0". */
const char* rtr_version(void);

/* Tuning knobs of this context (value 0 restores the automatic choice):
 *   "auto_graph"     1 (the default): rtr_recognize / rtr_recognize_learned /
 *                    rtr_recognize_host replay a repeated call from a CUDA
 *                    graph (see rtr_recognize); 0: every call enqueues its
 *                    kernels one by one;
 *   "icp_group"      lanes cooperating on one ICP source point's 1-NN search
 *                    (2, 4 or 8);
 *   "batch_workers"  workers (streams) of rtr_recognize_batch (1..16);
 *   "gc_window"      seeds per window of the grouping walk (32..1024);
 *   "gc_pass_lists"  1: the grouping keeps no pass lists, so a consensus
 *                    set that lost a member is recomputed by a new round
 *                    instead of in place by the walk (same clusters;
 *                    slower; 0 restores the default);
 *   "gc_inline"      sets the grouping walk recomputes in place per round
 *                    before it hands the rest of the window back to the
 *                    parallel phase (1..4096; default 16);
 *   "scene_grid_mm"  cell edge (mm) of the recognition's scene grid, used by
 *                    verification and ICP refinement (default: 1.5 x the ICP
 *                    distance; the table's size limit may widen it);
 *   "normals_grid_mm" cell edge (mm) of the scene normals' k-NN grid
 *                    (default: five voxel leaves);
 *   "scratch_limit_mb" the largest scratch arena the context may hold, in
 *                    MiB (0: no limit): a call needing more returns
 *                    RTR_ERR_OOM, as when cudaMalloc fails, and the arena
 *                    held so far stays usable.
 * Unknown keys or values return RTR_ERR_INVALID_ARG.  Results do not depend
 * on the knobs beyond FP32 summation order. */
rtr_status rtr_context_set_tuning(rtr_context* ctx, const char* key, int value);
/* The current value of a tuning knob (0 = the automatic choice). */
rtr_status rtr_context_get_tuning(const rtr_context* ctx, const char* key, int* value);

/* Create a context on `device`: owns a scratch arena, a device status word
 * and the tensor-map cache.  Fails with RTR_ERR_NO_DEVICE when the device is
 * not compute capability 10.3. */
rtr_status rtr_context_create(int device, rtr_context** out);
rtr_status rtr_context_destroy(rtr_context* ctx);
/* Grow the scratch arena to at least `bytes` (synchronises the device).  Call
 * before capturing a stream into a CUDA graph. */
rtr_status rtr_context_reserve(rtr_context* ctx, size_t bytes);
/* Bytes of scratch currently held. */
size_t rtr_context_scratch_bytes(const rtr_context* ctx);
/* Budget of every bounded device-side spin wait, in milliseconds (default 2000). */
rtr_status rtr_context_set_wait_budget_ms(rtr_context* ctx, double ms);
/* Synchronise `stream` and read (then clear) the device status word written by
 * persistent kernels (RTR_OK or RTR_ERR_TIMEOUT). */
rtr_status rtr_context_check(rtr_context* ctx, rtr_stream_t stream);

/* Stage profiling: when enabled, every rtr_* call records a CUDA event pair
 * around each of its stages ("grid_build", "icp_kernel", ...) on its stream.
 * After synchronising, rtr_context_profile_count/get read the recorded stages
 * in order (milliseconds) and rtr_context_profile_clear forgets them.  Keep
 * it off while capturing a graph. */
rtr_status rtr_context_set_profiling(rtr_context* ctx, int enabled);
int rtr_context_profile_count(rtr_context* ctx);
rtr_status rtr_context_profile_get(rtr_context* ctx, int i, const char** name, float* ms);
void rtr_context_profile_clear(rtr_context* ctx);
/* Kernels launched by this library in this process so far (all contexts). */
uint64_t rtr_launch_count(void);

/* ---- the reference's own GPU entry point (kept) --------------------------
 * Replaces kernel.cu:34-106 (declared at key_point.h:35-36).  Same signature,
 * same meaning: voxel_grid_occ is a HOST array of num_occ integer (x,y,z)
 * triples; voxel_grid_TDF is a HOST array of 27,000 floats.  For every voxel v
 * of the dim^3 grid (x fastest, then y, then z) it stores
 * min(900, min_i |v - occ_i|^2).  Synchronous; uses device 0.
 * Differences from kernel.cu, all on inputs where the reference misbehaves:
 *   - dim^3 > 27,000 or num_occ < 0 returns cudaErrorInvalidValue (the
 *     reference writes outside its 27,000-float device buffer);
 *   - at dim = 30 the reference's guard (kernel.cu:13) lets one thread write
 *     one float past the buffer; that write is not reproduced.  For dim < 30
 *     the same extra element (index dim^3, the voxel (0,0,dim)) lands inside
 *     the 27,000-float buffer and IS reproduced, so outputs match bit for bit.
 * Return type is cudaError_t in the reference; declared as int here so this
 * header does not need cuda_runtime.h (the values are cudaError_t codes). */
int ComputeTDFWithCuda(const int* voxel_grid_occ, float* voxel_grid_TDF,
                       int voxel_grid_dim, int num_occ);

/* Batched form of the above for many keypoints at once, device resident:
 * occupied voxels of keypoint k are d_occ[3*d_offsets[k] .. 3*d_offsets[k+1]),
 * output d_tdf[k*dim^3 .. (k+1)*dim^3).  d_offsets has n_keys+1 entries. */
rtr_status rtr_tdf_batch(rtr_context* ctx, const int* d_occ, const int* d_offsets,
                         int n_keys, int dim, float* d_tdf, rtr_stream_t stream);

/* ---- the reference's own descriptor route ---------------------------------
 * The occupancy / TDF / 36-yaw matcher of main (RealTimeRobot.cpp:56-108),
 * batched.  The reference builds a PCL octree per keypoint, per pair and per
 * rotation; here an octree with a defined box is a cube of 2^depth leaves
 * (leaf = integer key, depth-first order = Morton order with x the high bit),
 * with PCL's rules for sizing the cube and growing it when a point lands
 * outside (ceil((hi - lo - FLT_EPSILON) / res) leaves on the widest axis,
 * padded equally on both sides; growth adds a level, the old cube becoming
 * the upper half on every axis the point is not above; points are inserted
 * in ascending cloud index).  All calls synchronise the stream. */

/* KeyPoint::getOccupiedGrid (key_point.h:112-161) for n_keys keypoints over
 * one cloud: the points inside [key - half_box, key + half_box] (float box,
 * inclusive) as CSR d_offsets[n_keys + 1] / d_indices (ascending index), and
 * d_number[k] = Occupiedgrid.Number, the occupied leaves of edge resolution
 * in the octree of that box.  *h_total = the number of indices; when it
 * exceeds cap_indices the call returns RTR_ERR_CAPACITY with offsets and
 * numbers written (allocate and call again).  2 * half_box / resolution <= 30. */
rtr_status rtr_ref_occupancy(rtr_context* ctx, const float* d_cloud, int n, const float* d_keys,
                             int n_keys, float resolution, float half_box, int32_t* d_number,
                             int32_t* d_offsets, int32_t* d_indices, long long cap_indices,
                             long long* h_total, rtr_stream_t stream);

/* KeyPoint::get_TSDF (key_point.h:251-334): from each keypoint's occupancy
 * CSR, the occupied leaves of the +-half_tdf octree, the first in tree order
 * dropped, as integer voxels (centre - box corner) / resolution, then the
 * field of ComputeTDFWithCuda.  d_tdf: n_keys * dim^3 floats with
 * dim = (int)(half_tdf / resolution * 2) (30 at the defaults 0.01 / 0.15),
 * written to *h_dim.  A keypoint without occupied leaves gets 900
 * everywhere (the reference allocates a negative-size array there). */
rtr_status rtr_ref_tdf(rtr_context* ctx, const float* d_cloud, const float* d_keys, int n_keys,
                       const int32_t* d_offsets, const int32_t* d_indices, float resolution,
                       float half_tdf, float* d_tdf, int* h_dim, rtr_stream_t stream);

/* get_Distance (matching.h:122-222) for n_pairs (model keypoint, scan
 * keypoint) pairs, or for all n_model * n_scan pairs model-major when
 * d_pair_m and d_pair_s are NULL.  The model keypoint's occupancy cloud is
 * moved by (k - sk), turned 36 times by 10 degrees about the keypoint's
 * vertical axis (cumulatively, in float), and each time its occupied leaves
 * in the keypoint's field box (all but the first) read the field as
 * grid[y*30 + z*900 + x]; as in the reference, the squared field values are
 * added in float, leaf by leaf in the tree's depth-first order, into a
 * running score that no rotation resets, which is then divided by
 * (leaves - 1) in float; the lowest wins.  d_score[p] = that score,
 * d_T[16p] = the row-major 4x4 scale(kz/sz) * T(k) * Rz(best) * T(-k) *
 * T(k - sk).  Definitions where the reference is undefined: a field index
 * outside [0, 27000) reads 900; a cloud that would need more than 21 octree
 * levels, or a non-finite keypoint, gives score NaN and the identity.  The
 * field must be 30^3 (half_tdf / resolution = 15); occupancy clouds of up to
 * 8192 points whose rotated extent stays within 32 leaves (half_box <=
 * 0.106 m at 1 cm). */
rtr_status rtr_ref_distance(rtr_context* ctx, const float* d_mcloud, const float* d_mkeys,
                            int n_model, const int32_t* d_moffsets, const int32_t* d_mindices,
                            const float* d_mtdf, const float* d_skeys, int n_scan,
                            const int32_t* d_pair_m, const int32_t* d_pair_s, long long n_pairs,
                            float resolution, float half_tdf, float* d_score, float* d_T,
                            rtr_stream_t stream);

/* The all-pairs loop of main (RealTimeRobot.cpp:70-102): pair p = m * n_scan
 * + s is kept when d_score_all[p] < max_score (3 in main) and the gates of
 * function.h:158-178 pass as written: match_by_height passes unless the
 * ratio is NaN (float(2/3) is 0), match_by_area rejects a ratio above 3 or
 * below 0 (float(1/3) is 0) over the 3 plane areas per keypoint (d_*v3,
 * NULL = the KeyPoint default 0.16), match_by_occupied keeps
 * Number_m / Number_s (integer quotient) in [1, 2].  d_pair_idx gets the
 * kept p ascending; *h_n_pairs their number (RTR_ERR_CAPACITY above cap). */
rtr_status rtr_ref_correspond(rtr_context* ctx, const float* d_mkeys, const int32_t* d_mnumber,
                              const double* d_mv3, int n_model, const float* d_skeys,
                              const int32_t* d_snumber, const double* d_sv3, int n_scan,
                              const float* d_score_all, float max_score, int32_t* d_pair_idx,
                              int cap, int* h_n_pairs, rtr_stream_t stream);

/* Ransac (function.h:35-109) over the kept pairs: pair i's transform
 * (d_T_all[16 * p_i]) moves every kept pair's scan keypoint; pair j is an
 * inlier when |k_j - T sk_j| < inlier_dist (0.15; float distance) and
 * d_score_all[p_j] < max_des (100).  The first transform with the most
 * inliers wins: h_T (16 floats, row-major; identity when no pair has an
 * inlier, where the reference returns an uninitialised matrix), *h_inliers,
 * *h_best = its position in d_pair_idx or -1. */
rtr_status rtr_ref_ransac(rtr_context* ctx, const float* d_mkeys, int n_model, const float* d_skeys,
                          int n_scan, const int32_t* d_pair_idx, int n_pairs,
                          const float* d_score_all, const float* d_T_all, float inlier_dist,
                          float max_des, float* h_T, int* h_inliers, int* h_best,
                          rtr_stream_t stream);

/* ---- Harris3D keypoints -----------------------------------------------------
 * The detector of ModelPoint::getKeypoint / ScanPoint::getKeypoint
 * (model_point.h:127-136, scan_point.h:85-94: pcl::HarrisKeypoint3D with
 * radius 0.05, threshold 0.01, non-maximum suppression, refinement at its
 * default, on).  PCL is absent, so the operator is stated here: neighbours
 * are the points within `radius` (the point included), every sum in
 * ascending index order; normal = smallest eigenvector of the neighbours'
 * FP32 covariance; M = mean of n n^T over the neighbours' normals; response
 * R = det(M) - 0.04 tr(M)^2 + 0.04, which for unit normals is det(M): 0 on
 * faces and edges, up to 1/27 at a corner of three faces (the scale the
 * reference's 0.01 threshold fits).  Keypoints: R > threshold and (non_max)
 * no neighbour with a larger R.  Refinement moves each to the least-squares
 * intersection of the tangent planes of the points within `radius` (FP64),
 * at most 10 steps, while well conditioned and within `radius` of its
 * point.  d_keys: up to n x {x, y, z, R} in ascending point index; d_src
 * (optional): the keypoints' point indices; *d_count (device) = K.
 * A point with more than 1024 neighbours returns RTR_ERR_CAPACITY.
 * Synchronises.  Equal to the CPU oracle (oracle/harris.c) bit for bit. */
typedef struct rtr_harris_params {
  float radius;     /* 0.05 m */
  float threshold;  /* 0.01   */
  int   non_max;    /* 1      */
  int   refine;     /* 1      */
} rtr_harris_params;
void rtr_harris_default_params(rtr_harris_params* p);
rtr_status rtr_harris3d(rtr_context* ctx, const float* d_pts, int n, const rtr_harris_params* p, float* d_keys,
                        int32_t* d_src, int* d_count, rtr_stream_t stream);

/* ---- plane segmentation and the plane-area vector --------------------------
 * ModelPoint::getArea / ScanPoint::get_Area (model_point.h:170-245,
 * scan_point.h:117-188) and KeyPoint::get_Vector3D (key_point.h:87-111).
 * The reference uses PCL's SACSegmentation (RANSAC plane, 150 iterations,
 * 5 mm), ExtractIndices and ConvexHull: planes are taken out of the cloud one
 * after another while more than 15 % of the points remain.  Here:
 *   - points with a non-finite coordinate take no part;
 *   - RANSAC sample s of round r draws three positions in the remaining
 *     points from a SplitMix64 hash of (seed, r, s); repeated positions or
 *     collinear points skip the sample (at most 10 x max_iterations skips);
 *     the plane's score is its number of points within `distance` (float
 *     |n.p + d|); samples are taken in order until 99 % confidence (the
 *     adaptive count log(0.01) / log(1 - w^3)) or max_iterations valid
 *     ones; the first best wins;
 *   - the plane is refitted by least squares to its inliers (FP64 sums in a
 *     fixed order, smallest covariance eigenvector), and its inliers are
 *     selected again with the refitted plane (no inlier ends the loop);
 *   - area = the area of the 2-D convex hull of the inliers projected onto
 *     the plane; perimeter = that hull's perimeter (for a hull Qhull takes
 *     as two-dimensional, PCL's getTotalArea reports Qhull's "area", the
 *     perimeter);
 *   - is_vertical: 0 when the normal is within 10 degrees of z (is_h_plane),
 *     1 when within 80-100 degrees (is_v_plane), -1 otherwise; kept = the
 *     reference's surface list (horizontal or vertical, area >= min_area).
 * Results are bit-identical to the CPU oracle's (oracle/planes.c). */
typedef struct rtr_plane_params {
  int      max_iterations; /* 150                                         */
  float    distance;       /* inlier distance, 0.005 m                     */
  double   remain_frac;    /* stop when at most this fraction remains (0.15) */
  double   min_area;       /* surfaces kept from this area (0.16 m^2)      */
  uint64_t seed;           /* RANSAC samples (0)                           */
} rtr_plane_params;

typedef struct rtr_surface {
  double area;          /* hull area in the plane, m^2                    */
  double perimeter;     /* hull perimeter, m                              */
  float  coeffs[4];     /* a, b, c (unit normal), d: a x + b y + c z + d = 0 */
  int    is_vertical;   /* 0 horizontal, 1 vertical, -1 neither            */
  int    kept;          /* in the reference's surface list                 */
  int    n_inliers;
  int    hull_vertices;
  int    flat;          /* smallest / largest inlier covariance eigenvalue < 1e-3 */
  int    pad;
} rtr_surface;

void rtr_plane_default_params(rtr_plane_params* p);
/* Every extracted plane in order, kept or not, into h_surfaces (room for
 * max_surfaces; more planes return RTR_ERR_CAPACITY with the first
 * max_surfaces written); *h_n_surfaces = the number written.  Synchronises. */
rtr_status rtr_plane_segment(rtr_context* ctx, const float* d_pts, int n, const rtr_plane_params* p,
                             rtr_surface* h_surfaces, int max_surfaces, int* h_n_surfaces,
                             rtr_stream_t stream);
/* get_Vector3D for n_keys keypoints over the kept surfaces of h_surfaces,
 * in list order: the first horizontal surface within 5 cm gives v3[0], the
 * first two vertical ones within 2 cm give v3[1] and v3[2] (then sorted
 * descending); 0.16 where none.  The distance is getDistance's (key_point.h
 * :38-43): float expressions, sqrt of a float sum, divided in double.
 * d_v3: n_keys x 3 doubles, ready for rtr_ref_correspond's area gate.
 * Synchronises. */
rtr_status rtr_vector3d(rtr_context* ctx, const float* d_keys, int n_keys, const rtr_surface* h_surfaces,
                        int n_surfaces, double* d_v3, rtr_stream_t stream);

/* ---- nearest-neighbour search ---------------------------------------------
 * Exact searches over a radix-sorted uniform grid.  Squared distances are
 * computed in FP32 as ((dx*dx + dy*dy) + dz*dz) with dx = q.x - p.x, each
 * operation rounded separately (no fused multiply-add); ties go to the lowest
 * target index.  These are the rules of the CPU oracle, so indices are
 * bit-exact against it. */

/* 1-NN of each query among the targets with d^2 <= max_dist^2
 * (max_dist <= 0 or infinite: unbounded).  Writes the target index or -1 and
 * the squared distance (or +inf). */
rtr_status rtr_knn1(rtr_context* ctx, const float* d_query, int n_query,
                    const float* d_target, int n_target, float max_dist,
                    int32_t* d_out_idx, float* d_out_d2, rtr_stream_t stream);

/* rtr_knn1 without any allocation, for callers that may not allocate device
 * memory (a real-time control loop with a fixed memory budget, a caller that
 * owns every allocation itself, code running where cudaMalloc would
 * synchronise the device).  No counterpart in the reference.
 *
 * Same arguments and results as rtr_knn1 (bit-identical outputs), minus the
 * context: it runs on the calling thread's current device.  Its grid lives in
 * one fixed device array of about 7 MiB compiled into the library, so
 * n_target is limited to RTR_KNN1_STATIC_MAX_TARGET (larger sets return
 * RTR_ERR_CAPACITY before anything is launched; use rtr_knn1 for those).
 * n_query is not limited.  Nothing in the array needs to start at zero:
 * each call rebuilds every part it reads.
 *
 * The first call on a device looks up the array's address
 * (cudaGetSymbolAddress), which may load the module; make that first call
 * before capturing a stream.  The address is kept for the life of the
 * process, so calls after cudaDeviceReset on that device are not supported.
 * Every buffer must be device (or managed) memory of the current device;
 * others return RTR_ERR_INVALID_ARG before any launch.  The array is shared
 * by every call on a device:
 * two calls whose work overlaps in time (different streams, or different
 * host threads, without ordering between them) race and both may return wrong
 * indices.  Order them on one stream or with events. */
#define RTR_KNN1_STATIC_MAX_TARGET 65536
rtr_status rtr_knn1_static(const float* d_query, int n_query, const float* d_target,
                           int n_target, float max_dist, int32_t* d_out_idx,
                           float* d_out_d2, rtr_stream_t stream);

/* k nearest neighbours (1 <= k <= 32), sorted by (d^2, index).  Unbounded. */
rtr_status rtr_knn(rtr_context* ctx, const float* d_query, int n_query,
                   const float* d_target, int n_target, int k,
                   int32_t* d_out_idx, float* d_out_d2, rtr_stream_t stream);

/* Fixed-radius and box searches: for each query, every target with
 * d^2 <= radius^2 (rtr_radius_search; d^2 as above), or every target inside
 * the axis-aligned box [q - h, q + h] with the bounds formed in FP32 and
 * included (rtr_box_search; the box of OctreePointCloudSearch::boxSearch in
 * KeyPoint::getOccupiedGrid, key_point.h:118-140), in ascending target index.
 * d_out_count[q] (optional) receives the true count; d_out_idx[q *
 * max_per_query ...] the first max_per_query indices (the lowest ones when
 * the count is larger), the slots past the count -1.  max_per_query = 0
 * counts only (d_out_idx may then be NULL).  Queries or targets with a
 * non-finite coordinate never match.  radius / half extent: finite, >= 0. */
rtr_status rtr_radius_search(rtr_context* ctx, const float* d_query, int n_query,
                             const float* d_target, int n_target, float radius,
                             int max_per_query, int32_t* d_out_idx, int32_t* d_out_count,
                             rtr_stream_t stream);
rtr_status rtr_box_search(rtr_context* ctx, const float* d_query, int n_query,
                          const float* d_target, int n_target, float half_extent,
                          int max_per_query, int32_t* d_out_idx, int32_t* d_out_count,
                          rtr_stream_t stream);

/* Inlier counts of candidate poses (the recognition's hypothesis score,
 * exported): for each of the n_poses model -> scene poses (row-major 4x4
 * doubles on the device, applied in FP32 as ((r0 x + r1 y) + r2 z) + t), the
 * number of model points with a scene point within radius (d^2 <= radius^2
 * as above).  d_counts[n_poses] on the device.  radius: finite, > 0. */
rtr_status rtr_pose_inliers(rtr_context* ctx, const float* d_model, int n_model,
                            const float* d_scene, int n_scene, const double* d_poses,
                            int n_poses, float radius, int32_t* d_counts, rtr_stream_t stream);

/* ---- ICP (point-to-point) -------------------------------------------------
 * Replaces the PCL IterativeClosestPoint of keyPointICP (function.h:111-148).
 * One persistent cooperative kernel runs all iterations: per iteration it
 * transforms the source, finds the exact 1-NN in the target grid, rejects
 * pairs beyond max_corr_dist, accumulates the centred 3x3 cross-covariance in
 * FP32 with compensated (Kahan) sums, reduces the block partials in FP64 and
 * solves the pose in FP64 (Umeyama, Jacobi SVD). */
typedef struct rtr_icp_params {
  int    max_iterations;         /* PCL default 10                                */
  float  max_corr_dist;          /* metres; <= 0 = unbounded (PCL default)        */
  double transformation_epsilon; /* stop when |dt|^2 < eps (0: only dt == 0)       */
  double rotation_epsilon;       /* stop when cos(dangle) > this (0: disabled)     */
  float  cell_size;              /* target grid cell; 0 = automatic               */
  int    record_trace;           /* fill d_trace_pose / d_trace_corr if non-NULL  */
} rtr_icp_params;

typedef struct rtr_icp_result {
  double pose[16];     /* final source->target transform, row-major          */
  double fitness;      /* mean squared distance of the last correspondences  */
  int    iterations;   /* iterations performed                               */
  int    converged;    /* 1 unless stopped for < 3 correspondences / timeout */
  int    n_corr;       /* correspondences of the last iteration              */
  int    status;       /* RTR_OK or RTR_ERR_TIMEOUT                          */
} rtr_icp_result;

void rtr_icp_default_params(rtr_icp_params* p);

/* h_init_pose: host row-major 4x4 (NULL = identity).  d_result: device
 * rtr_icp_result.  d_trace_pose (optional): (max_iterations+1)*16 doubles —
 * the pose before every iteration and after the last.  d_trace_corr
 * (optional): max_iterations*n_src int32 — the target index (or -1) of every
 * source point (original order) in every iteration. */
rtr_status rtr_icp(rtr_context* ctx, const float* d_src, int n_src,
                   const float* d_tgt, int n_tgt, const rtr_icp_params* params,
                   const double* h_init_pose, rtr_icp_result* d_result,
                   double* d_trace_pose, int32_t* d_trace_corr, rtr_stream_t stream);

/* Same with HOST point buffers and a HOST result; copies in and out and
 * synchronises.  This is the call keyPointICP makes. */
rtr_status rtr_icp_host(rtr_context* ctx, const float* h_src, int n_src,
                        const float* h_tgt, int n_tgt, const rtr_icp_params* params,
                        const double* h_init_pose, rtr_icp_result* h_result);

/* Independent ICP problems of one source against one target, each from its
 * own initial pose (d_init_poses: n_problems row-major 4x4 doubles on the
 * device; NULL: identity), in one persistent launch over one target grid:
 * the multi-hypothesis refinement of the recognition, exported.  params as
 * rtr_icp (record_trace ignored); d_results[k] receives problem k's result.
 * n_problems: 1 .. the co-resident block count (a few hundred); the source
 * is used in its given order. */
rtr_status rtr_icp_multi(rtr_context* ctx, const float* d_src, int n_src, const float* d_tgt,
                         int n_tgt, const rtr_icp_params* params, const double* d_init_poses,
                         int n_problems, rtr_icp_result* d_results, rtr_stream_t stream);

/* Where the last ICP launch of the context spent its time (first problem of
 * the launch, summed over iterations, nanoseconds): [0] block 0's search and
 * block sums, [1] the last-arriving block's serial section (cross-block
 * reduction, pose solve, release), [2] block 0's wait for the release, [3]
 * iterations, [4] and [5] the serial section up to the end of its
 * cross-block reduction and of its pose solve.  Synchronises. */
rtr_status rtr_icp_stats(rtr_context* ctx, long long* h_stats6);

/* ---- recognition stages --------------------------------------------------
 * The reference computes these inside ModelPoint/ScanPoint::getKeypoint
 * (model_point.h:99-156, scan_point.h:57-113: PCL normals + keypoints) and
 * KeyPoint (key_point.h:112-161, 251-334: octree voxels + local descriptor).
 * Counts written to d_count are device ints, so calls can be chained without
 * a host round trip. */

/* Voxel-grid filter (PCL VoxelGrid semantics): voxel of p = floor(p / leaf)
 * per axis (FP32, p * (1/leaf)); one centroid per occupied voxel, in
 * ascending voxel key (x fastest); centroid = FP32 sum of the voxel's points
 * in ascending input index divided by the count.  d_out holds n points;
 * *d_count = number of voxels, or -1 when the key space exceeds 2^32. */
rtr_status rtr_voxel_downsample(rtr_context* ctx, const float* d_pts, int n, float leaf,
                                float* d_out, int* d_count, rtr_stream_t stream);

/* Uniform sampling (PCL UniformSampling): per voxel of edge `radius`, the
 * index of the point nearest the voxel centre ((floor(p / r) + 0.5) * r),
 * ties to the lowest index; in ascending voxel key.  d_idx holds n. */
rtr_status rtr_uniform_sample(rtr_context* ctx, const float* d_pts, int n, float radius,
                              int32_t* d_idx, int* d_count, rtr_stream_t stream);

/* Normals (PCL NormalEstimation with k neighbours incl. the point): FP32 mean
 * and centred covariance in kNN order, exact Jacobi eigen-solve, the smallest
 * eigenvector flipped towards h_vp3, curvature = l0 / (l0 + l1 + l2).
 * d_normals: n x {nx, ny, nz, curvature}.  k in {8, 10, 16}.  search_cell:
 * grid edge hint for the kNN search (0 = automatic). */
rtr_status rtr_normals(rtr_context* ctx, const float* d_pts, int n, int k, const float* h_vp3,
                       float search_cell, float* d_normals, rtr_stream_t stream);

/* Outward orientation for a full (360 degree) model cloud, where no single
 * viewpoint sees every face: each normal is flipped towards the side whose
 * cylinder (radius rc, axial distance in (gap, len]) holds fewer points. */
rtr_status rtr_orient_normals_outward(rtr_context* ctx, const float* d_pts, float* d_normals,
                                      int n, float rc, float gap, float len,
                                      rtr_stream_t stream);

/* SHOT-style 352-d descriptor (Tombari, Salti, Di Stefano 2010) at keypoints
 * d_keys (indices into d_pts): 2 radial x 2 elevation x 8 azimuth volumes x
 * 11 bins of cos(normal, z), quadrilinear interpolation, L2 normalised.
 * Support: points within `radius` facing the keypoint's side
 * (n_j . n_k >= -0.2).  LRF: weighted-covariance eigenvectors (x largest, z
 * smallest), x signed by the majority rule, z by agreement with the support's
 * oriented normals.  d_desc: nk x 352; d_lrf (optional): nk x 9 (rows x,y,z).
 * Deterministic: the support's sums are fixed-point, so the result does not
 * depend on the order of the points.  radius: 1e-6 to 1e6 (RTR_ERR_INVALID_ARG
 * outside). */
rtr_status rtr_shot352(rtr_context* ctx, const float* d_pts, const float* d_normals, int n,
                       const int32_t* d_keys, int nk, float radius, float* d_desc,
                       float* d_lrf, rtr_stream_t stream);

/* Descriptor 1-NN on the tensor cores (the all-pairs loop of
 * RealTimeRobot.cpp:73-102, recast as SHOT 1-NN): BF16 (hi + lo split)
 * tcgen05 GEMM with FP32 accumulation, per-query top-8, exact FP32 re-rank and
 * a certified error bound.  Uncertified queries (near-ties: flat faces give
 * many near-equal descriptors) take a second GEMM pass that lists every row
 * within the tie margin, and the exact minimum over that band; a band over
 * 256 rows falls back to an exact scan of the whole database.  The indices
 * and distances equal rtr_match_exact's bit for bit. */
rtr_status rtr_match(rtr_context* ctx, const float* d_query, int n_query, const float* d_db,
                     int n_db, int32_t* d_idx, float* d_d2, rtr_stream_t stream);
/* Queries of the last tensor-core match whose top-8 could not be certified
 * (re-scanned exactly).  Synchronises the device. */
rtr_status rtr_match_stats(rtr_context* ctx, int* h_uncertified);
/* The same, and how many of them needed the exact scan of the whole
 * database.  Synchronises the device. */
rtr_status rtr_match_stats_ex(rtr_context* ctx, int* h_uncertified, int* h_full_scans);

/* Exact FP32 1-NN of 352-d descriptors: d^2 = sum over k in order of
 * (a_k - b_k)^2, each op rounded separately, ties to the lowest index. */
rtr_status rtr_match_exact(rtr_context* ctx, const float* d_query, int n_query,
                           const float* d_db, int n_db, int32_t* d_idx, float* d_d2,
                           rtr_stream_t stream);

/* Geometric-consistency grouping (Chen & Bhanu 2007, PCL
 * GeometricConsistencyGrouping), which takes the place of the reference's
 * pair-consensus loop (Ransac, function.h:35-109).  Correspondence i pairs
 * model keypoint d_corr_m[i] with scene keypoint d_corr_s[i] at descriptor
 * distance d_corr_d[i].  Correspondences are taken in ascending distance
 * (ties: input order); each not-yet-taken one seeds a set that admits, in the
 * same order, every not-taken correspondence whose model-side and scene-side
 * distances to every member differ by at most gc_size; a set with at least
 * gc_thresh members becomes a cluster and its members are taken.  Outputs, for
 * the first max_clusters clusters: members (original correspondence indices,
 * max_members per row, -1 padded), sizes, and the least-squares model->scene
 * pose (row-major 4x4, FP64).  The walk runs on the device in one cooperative
 * launch; the call synchronises once, to return the cluster count.  A set
 * may hold every correspondence while n_corr^2 ints fit in 128 MiB (n_corr
 * up to 5,792); above that, sets longer than 128 MiB / (4 n_corr) members
 * (at least 128), or more than 1,441,792 correspondences, return
 * RTR_ERR_CAPACITY.  A cluster longer than max_members keeps its first
 * max_members members in d_members; d_sizes and the pose cover all of them. */
rtr_status rtr_gc_group(rtr_context* ctx, const float* d_model_kp, const float* d_scene_kp,
                        const int32_t* d_corr_m, const int32_t* d_corr_s, const float* d_corr_d,
                        int n_corr, float gc_size, int gc_thresh, int max_clusters,
                        int max_members, int32_t* d_members, int32_t* d_sizes,
                        double* d_poses, int* h_n_clusters, rtr_stream_t stream);
/* Work of the last grouping on this context: h_stats8[0] = rounds of the
 * window/walk loop, [1] = position where the walk ended, [2] = consensus
 * sets computed (including recomputations), [3..6] = microseconds spent in
 * the round phases (seed selection, seed tests, admission, walk; barrier
 * waits included), [7] = candidates that passed a seed test, summed over the
 * computed sets.  No synchronisation. */
rtr_status rtr_gc_stats(rtr_context* ctx, int* h_stats8);

/* ---- recognition pipeline ------------------------------------------------
 * The whole chain of main (RealTimeRobot.cpp:39-105) for one known object
 * model and one scene: voxel filter -> normals -> uniform keypoints ->
 * SHOT-352 -> 1-NN descriptor matching -> geometric-consistency grouping ->
 * hypothesis verification (the role of Ransac, function.h:35-109: every
 * cluster's pose is scored by the fraction of model points landing within
 * hv_inlier_r of the scene) -> ICP refinement of the refine_top best
 * hypotheses in one batched persistent launch -> final score (fraction of
 * model voxels within accept_inlier_r) -> non-maximum suppression. */
#define RTR_MAX_INSTANCES 16

typedef struct rtr_recog_params {
  float voxel_leaf;             /* 0.01 m                                        */
  int   normal_k;               /* 10                                            */
  float scene_keypoint_r;       /* uniform sampling of the scene, 0.02 m         */
  float model_keypoint_r;       /* uniform sampling of the model, 0.02 m         */
  float descriptor_r;           /* SHOT support radius, 0.04 m                   */
  float match_max_d2;           /* keep a match when d^2 < this (0.25)           */
  float gc_size;                /* consistency bin, 0.01 m                       */
  int   gc_thresh;              /* minimum cluster size, 5                       */
  int   max_clusters;           /* hypotheses kept from grouping (<= 256)        */
  float hv_inlier_r;            /* hypothesis score radius, 0.02 m               */
  int   hv_subsample;           /* score every hv_subsample-th model voxel (4)    */
  int   refine_top;             /* hypotheses refined by ICP (<= 64)             */
  int   icp_iterations;         /* 30                                            */
  float icp_max_dist;           /* 0.02 m                                        */
  float accept_inlier_r;        /* final score radius, 0.01 m                    */
  float accept_score;           /* instances need at least this final score      */
  float nms_dist;               /* refined poses closer than this are one object */
  int   max_instances;          /* <= RTR_MAX_INSTANCES                           */
  float viewpoint[3];           /* scene sensor origin (normal orientation)      */
  float keypoint_min_curvature; /* curvature gate on scene keypoints (0 = off)   */
  int   scene_outward;          /* 1: the scene is a full object segment; orient  */
                                /* its normals outward like a model's            */
} rtr_recog_params;

typedef struct rtr_instance {
  double pose[16];   /* model -> scene, row-major */
  float  score;      /* final inlier fraction     */
  int    hypothesis; /* grouping cluster index    */
  int    cluster_size;
  int    pad;
} rtr_instance;

typedef struct rtr_recog_result {
  int n_instances;
  int n_voxels;          /* scene voxels        */
  int n_keypoints;       /* scene keypoints     */
  int n_correspondences;
  int n_clusters;
  int status;            /* RTR_OK or RTR_ERR_NOT_FOUND */
  int pad[2];
  rtr_instance inst[RTR_MAX_INSTANCES];
} rtr_recog_result;

typedef struct rtr_model rtr_model;

void rtr_recog_default_params(rtr_recog_params* p);
/* Model preparation (the model side of main, RealTimeRobot.cpp:39-41,
 * 62-69): voxel filter, normals oriented outward, uniform keypoints, SHOT.
 * Device points in; the model owns its device buffers.  Synchronises. */
rtr_status rtr_model_create(rtr_context* ctx, const float* d_pts, int n,
                            const rtr_recog_params* p, rtr_model** out);
rtr_status rtr_model_destroy(rtr_model* m);
rtr_status rtr_model_info(const rtr_model* m, int* n_voxels, int* n_keypoints);
/* Device views of the model's buffers (any output may be NULL). */
rtr_status rtr_model_buffers(const rtr_model* m, const float** d_vox, const float** d_normals,
                             const int32_t** d_keys, const float** d_kp, const float** d_desc);
/* Recognise the model in a scene (device points).  d_result: device
 * rtr_recog_result.  Does not synchronise: every count stays on the device
 * and errors reach the context status word (rtr_context_check).  The first
 * call at a scene size may grow the context's scratch (that synchronises);
 * after it, calls of at most that size can be captured into a CUDA graph.
 * Such a graph holds the scratch's address: a later call that grows the
 * scratch (a larger scene, the learned form) moves it, and the graph must not
 * be launched again (rtr_context_reserve the largest size first).
 * The context does this itself for a repeated call ("auto_graph", on by
 * default): when a call repeats the previous one's model, scene and result
 * addresses, n and parameters (the scene's contents may change), the second
 * such call captures its launches into a CUDA graph and later ones replay
 * it, with the same results; any other call, a tuning change or a grown
 * scratch arena ends the replay.  Not while profiling or while the caller's
 * stream is itself being captured. */
rtr_status rtr_recognize(rtr_context* ctx, const rtr_model* model, const float* d_scene, int n,
                         const rtr_recog_params* p, rtr_recog_result* d_result,
                         rtr_stream_t stream);
/* Recognition with learned keypoint pruning (the "learned" form): after the
 * SHOT stage, `mlp` scores every scene keypoint's descriptor and only the
 * ceil(keep * K) most credible keypoints (ties: lower keypoint index) go on to
 * matching, in their original order; the rest is rtr_recognize's chain.
 * keep in (0, 1] (0.25 keeps the top quarter). */
rtr_status rtr_recognize_learned(rtr_context* ctx, const rtr_model* model, const rtr_mlp* mlp, float keep,
                                 const float* d_scene, int n, const rtr_recog_params* p,
                                 rtr_recog_result* d_result, rtr_stream_t stream);
/* ---- batched registration (many model x segment pairs) ---------------------
 * The pairs run concurrently: a pool of worker threads, each with a child
 * context and its own stream, takes the pairs largest first and runs the
 * recognition chain on each (rtr_recognize, or rtr_recognize_learned when
 * mlp is not NULL).  One host thread enqueues every pair: each worker is a
 * child context with its own stream, forked from and joined back to the
 * context's stream.  Result i (device, d_results[i]) is what the
 * single-pair call gives, except that each worker's cooperative kernels use a
 * share of the GPU: an ICP problem split over fewer blocks rounds its FP32
 * block sums differently (poses agree within 1e-5).  The number of workers is the context's
 * "batch_workers" tuning knob (default 4; see rtr_batch_autotune).  A model
 * may appear in several pairs.  Synchronises; the caller's inputs must be
 * complete when it is called (it synchronises the device first). */
typedef struct rtr_batch_pair {
  const rtr_model* model;
  const float* d_scene;   /* n points, 16-byte aligned */
  int n;
} rtr_batch_pair;
rtr_status rtr_recognize_batch(rtr_context* ctx, const rtr_batch_pair* h_pairs, int n_pairs,
                               const rtr_recog_params* p, const rtr_mlp* mlp, float keep,
                               rtr_recog_result* d_results);
/* The same batch captured once into a CUDA graph: create runs the batch once
 * (sizing every worker's scratch), then records its enqueue sequence; each
 * launch replays it on `stream` and returns without synchronising (check the
 * results after synchronising; rtr_context_check on the workers is not
 * needed: errors also leave a non-OK status in each result).  The scenes
 * must stay at the same device addresses; their contents, and the model
 * buffers' contents, may change between launches (same sizes).  The graph
 * also holds the addresses of the context's and its workers' scratch: a
 * later call on the context that needs more scratch (a larger batch, the
 * learned form after a plain graph) reallocates it, and launch then returns
 * RTR_ERR_INVALID_ARG instead of running; create the largest graphs first,
 * or size the scratch with the largest batch before creating any.  Destroy
 * a graph before its context. */
typedef struct rtr_batch_graph rtr_batch_graph;
rtr_status rtr_batch_graph_create(rtr_context* ctx, const rtr_batch_pair* h_pairs, int n_pairs,
                                  const rtr_recog_params* p, const rtr_mlp* mlp, float keep,
                                  rtr_recog_result* d_results, rtr_batch_graph** out);
rtr_status rtr_batch_graph_launch(rtr_batch_graph* g, rtr_stream_t stream);
rtr_status rtr_batch_graph_destroy(rtr_batch_graph* g);
/* Autotuner of the batch: times it under each (workers 1/2/4/8: pairs per
 * stream, the share of the GPU each pair's kernels get) x (ICP lanes per
 * source point 2/4/8) setting, then, with the fastest fixed, each scene-grid
 * cell of the verification and refinement searches (automatic, 20, 40,
 * 60 mm) and each normals k-NN grid cell (automatic, 20, 30, 80 mm); keeps
 * the fastest in the context's tuning knobs (rtr_context_get_tuning reads
 * them) and reports workers / ICP lanes in h_workers / h_icp_group (either
 * may be NULL).  The searches are exact, so the knobs change speed, not
 * results (beyond FP32 block-sum order in ICP).  Runs the batch 40 times;
 * d_results holds the last run's results. */
rtr_status rtr_batch_autotune(rtr_context* ctx, const rtr_batch_pair* h_pairs, int n_pairs,
                              const rtr_recog_params* p, const rtr_mlp* mlp, float keep,
                              rtr_recog_result* d_results, int* h_workers, int* h_icp_group);

/* Several models in one scene (the streaming workload's per-frame form):
 * the scene's stages (voxels, normals, keypoints, descriptors and, with mlp,
 * learned pruning) run once; each model's matching, grouping, verification
 * and refinement run on a worker stream ("batch_workers" knob, at most
 * n_models workers; one worker runs them in turn on `stream`).  Result i
 * (device, d_results[i]) is rtr_recognize(_learned) of h_models[i], up to the
 * FP32 rounding of ICP block sums when the workers share the GPU.
 * Synchronises and reports the workers' status words. */
rtr_status rtr_recognize_multi(rtr_context* ctx, const rtr_model* const* h_models, int n_models,
                               const rtr_mlp* mlp, float keep, const float* d_scene, int n,
                               const rtr_recog_params* p, rtr_recog_result* d_results,
                               rtr_stream_t stream);

/* Same with a HOST scene and a HOST result (copies in and out). */
rtr_status rtr_recognize_host(rtr_context* ctx, const rtr_model* model, const float* h_scene, int n,
                              const rtr_recog_params* p, rtr_recog_result* h_result);

/* ---- learned keypoint credibility ------------------------------------------
 * A small MLP scores each keypoint's SHOT-352 descriptor (352 -> 128 -> 64 ->
 * 1, ReLU, ReLU, sigmoid) so that low-credibility keypoints can be dropped
 * before matching.  No counterpart in the reference, whose README names the
 * problem.  Parameters (RTR_MLP_PARAMS floats, in this order): W1[128][352],
 * b1[128], W2[64][128], b2[64], w3[64], b3.  Forward passes use the weight
 * matrices rounded to BF16 and accumulate in FP32; training is Adam (beta1
 * 0.9, beta2 0.999, eps 1e-8) on the mean binary cross-entropy of the logit,
 * with gradients taken for the FP32 master weights. */
#define RTR_MLP_PARAMS 53505
/* h_params: RTR_MLP_PARAMS floats, or NULL for a seeded He-uniform start
 * (zero biases).  Synchronises. */
rtr_status rtr_mlp_create(rtr_context* ctx, const float* h_params, uint64_t seed, rtr_mlp** out);
rtr_status rtr_mlp_destroy(rtr_mlp* m);
/* FP32 master weights to / from the host (setting them resets Adam). */
rtr_status rtr_mlp_get_params(const rtr_mlp* m, float* h_params);
rtr_status rtr_mlp_set_params(rtr_mlp* m, const float* h_params);
/* Credibility in (0, 1) of n descriptors (device [n][352] -> device [n]). */
rtr_status rtr_mlp_score(rtr_context* ctx, const rtr_mlp* m, const float* d_x, int n, float* d_score,
                         rtr_stream_t stream);
/* Mean loss and its gradient (RTR_MLP_PARAMS floats, device) on n labelled
 * rows (labels 0 or 1, device [n]); no update. */
rtr_status rtr_mlp_loss_grad(rtr_context* ctx, const rtr_mlp* m, const float* d_x, const float* d_y, int n,
                             float* d_grad, float* d_loss, rtr_stream_t stream);
/* One Adam step on the n rows given. */
rtr_status rtr_mlp_train_step(rtr_context* ctx, rtr_mlp* m, const float* d_x, const float* d_y, int n, float lr,
                              float* d_loss, rtr_stream_t stream);
/* Minibatch training: `epochs` passes over the n rows in a seeded shuffled
 * order, batches of `batch` rows.  h_epoch_loss (optional, `epochs` floats)
 * receives the row-weighted mean batch loss of each epoch.  Synchronises. */
rtr_status rtr_mlp_train(rtr_context* ctx, rtr_mlp* m, const float* d_x, const float* d_y, int n, int batch,
                         int epochs, float lr, uint64_t seed, float* h_epoch_loss);

/* ---- streaming: depth frames, back-projection, fusion map ------------------
 * Depth frames are organised width x height float32 images of z in metres
 * (0 = no return), pinhole (fx, fy, cx, cy).  A pose maps camera
 * coordinates (x right, y down, z forward) to world coordinates (row-major
 * 4x4, FP64 on the host). */

/* Points of a depth frame with min_z < z < max_z, in pixel order (row by
 * row), as world points pose * ((u - cx) z / fx, (v - cy) z / fy, z), each
 * operation rounded in FP32 (h_pose16 NULL = identity).  d_points holds
 * width * height points; the count goes to the device int d_count.
 * Synchronises (the pose is staged from the host). */
rtr_status rtr_depth_to_points(rtr_context* ctx, const float* d_depth, int width, int height, float fx,
                               float fy, float cx, float cy, const double* h_pose16, float min_z,
                               float max_z, float* d_points, int* d_count, rtr_stream_t stream);

/* Fusion map: a GPU hash table of voxels (edge `voxel`) keeping, per voxel,
 * its point count and the mean of its points.  Sums are kept in fixed point
 * (2^-40 m) with integer atomics, so the contents do not depend on the order
 * in which points arrive.  capacity is rounded up to a power of two and
 * should be at least twice the voxels the map will hold: an insert looks at
 * no more than 256 slots, and a point that finds none free is dropped and
 * makes rtr_map_extract return RTR_ERR_CAPACITY. */
typedef struct rtr_map rtr_map;
rtr_status rtr_map_create(rtr_context* ctx, int capacity, float voxel, rtr_map** out);
rtr_status rtr_map_destroy(rtr_map* m);
rtr_status rtr_map_clear(rtr_map* m, rtr_stream_t stream);
/* Adds the first *d_n (d_n NULL: n_cap) points (device). */
rtr_status rtr_map_integrate(rtr_map* m, const float* d_points, int n_cap, const int* d_n, rtr_stream_t stream);
/* Occupied voxels as {mean x, mean y, mean z, count (int bits)} into d_out
 * (in table order), their number into *h_count; with more than max_out
 * voxels only the count is written.  Synchronises. */
rtr_status rtr_map_extract(rtr_context* ctx, rtr_map* m, float* d_out, int max_out, int* h_count);

/* ---- synthetic inputs (host only; seeded, identical on every machine) ----- */

/* Shapes: 0 = chair (seat 0.45x0.45x0.03, four legs 0.03x0.03x0.45, backrest
 * 0.45x0.03x0.45), 1 = desk (top 1.2x0.6x0.03 on four 0.05x0.05x0.72 legs),
 * 2 = sofa (2.0x0.9x0.8 box assembly).  n points area-uniform on the boxes'
 * faces, floor at z = 0. */
rtr_status rtr_synth_shape(int shape, uint64_t seed, int n, float* h_out_xyz4);
/* Rigid transform: rotation axis uniform on the sphere, angle uniform in
 * [0, max_angle_deg], translation uniform in [-max_t, max_t] per axis. */
void rtr_synth_rigid(uint64_t seed, double max_angle_deg, double max_t, double* h_T16);
/* out = T * in + N(0, sigma^2) per coordinate (in and out may alias). */
void rtr_synth_transform_noise(const float* h_in, int n, const double* h_T16, double sigma,
                               uint64_t seed, float* h_out);
/* Remove a fraction U[0, max_frac] of the points on one side of a random
 * plane; writes the kept points in their original order, returns their count. */
int rtr_synth_crop(const float* h_in, int n, double max_frac, uint64_t seed, float* h_out);

/* One viewpoint of a 5 x 5 x 3 m room (floor z = 0, walls y = +2.5 and
 * x = -2.5) holding box furniture at seeded yaw and position, ray-cast from a
 * pinhole camera: each point is the first hit of a ray through a uniformly
 * drawn pixel, plus N(0, sigma^2) noise per coordinate. */
typedef struct rtr_room_params {
  int    n_points;               /* 300,000                               */
  int    n_chairs, n_desks, n_sofas;
  double sigma;                  /* 0.003 m                               */
  double cam[3];                 /* (0, -2.5, 1.5)                        */
  double look_at[3];             /* (0, 0.8, 0.3)                         */
  int    width, height;          /* 640 x 480                             */
  double fx, fy, cx, cy;         /* 400, 400, 319.5, 239.5                */
} rtr_room_params;
void rtr_room_default_params(rtr_room_params* p);
/* h_inst_shape / h_inst_pose16 (optional, max_instances entries): each piece's
 * shape id and object->world pose (row-major 4x4). */
rtr_status rtr_synth_room(const rtr_room_params* p, uint64_t seed, float* h_out_xyz4,
                          int max_instances, int* h_inst_shape, double* h_inst_pose16,
                          int* h_n_instances);
/* The furniture of the same room (same placement rule) as world boxes: 12
 * floats per box {cos yaw, sin yaw, x, y, lo[3], hi[3], shape, instance}
 * (lo/hi in the object frame). */
rtr_status rtr_synth_room_boxes(const rtr_room_params* p, uint64_t seed, float* h_boxes12, int max_boxes,
                                int* h_n_boxes, int* h_inst_shape, double* h_inst_pose16,
                                int max_instances, int* h_n_instances);
/* A smooth seeded camera path through the room at `fps`: x sweeps +-1.2 m
 * (peak 0.5 m/s) near y = -2.3 at 1.5 m height, yaw +-20 deg (peak
 * 17.5 deg/s), 25 deg down.  Poses camera -> world, 16 doubles per frame. */
void rtr_synth_trajectory(uint64_t seed, int n_frames, double fps, double* h_poses16);
/* Ray-cast depth frames of a room (floor, two walls, the boxes) from the
 * given camera poses into d_depth (n_frames x height x width), with
 * N(0, (noise_k z^2)^2) depth noise from a counter-based hash of (seed, frame,
 * pixel).  On the GPU; synchronises. */
rtr_status rtr_synth_depth_frames(rtr_context* ctx, const float* h_boxes12, int n_boxes,
                                  const double* h_poses16, int n_frames, int width, int height, float fx,
                                  float fy, float cx, float cy, float noise_k, uint64_t seed, float* d_depth,
                                  rtr_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* RTR_H_ */

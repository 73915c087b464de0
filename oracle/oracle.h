/*
 * oracle.h — CPU restatement of the registration hot path, used ONLY as the
 * checker (tests/, __graft_entry__.smoke) and as the timed CPU baseline
 * (bench.py cpu_baseline / --impl reference).  Never linked into librtr.so.
 *
 * Parity status: the PCL-backed stages (1-NN, ICP, voxel grid, normals,
 * uniform sampling, SHOT, matching, GC) restate published methods because PCL
 * 1.8.0's source is not part of the reference; they are pinned only by the
 * reference's recorded PCD fixtures (translation pairs, see tests/golden).  The
 * TDF restates kernel.cu:8-31 exactly.  refmatch.c restates the reference's
 * own descriptor route (getOccupiedGrid, get_TSDF, get_Distance, the gates,
 * Ransac) over PCL's octree rules; against PCL itself it is unpinned.
 *
 * Arithmetic rules shared with the GPU (compile with -ffp-contract=off):
 *   d2(q, p)  = ((dx*dx + dy*dy) + dz*dz), dx = q.x - p.x, each op rounded;
 *   T(p).x    = ((r00*x + r01*y) + r02*z) + t0 with r, t rounded to float;
 *   ties      = lowest target index.
 */
#ifndef RTR_ORACLE_H_
#define RTR_ORACLE_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

int orc_num_threads(void);
void orc_set_threads(int n);

/* ---- nearest neighbours (PCL KdTreeFLANN nearestKSearch semantics, made exact) */
void orc_nn1_brute(const float* q, int nq, const float* t, int nt, float r2max, int32_t* idx,
                   float* d2);
void orc_nn1_grid(const float* q, int nq, const float* t, int nt, float r2max, float cell,
                  int32_t* idx, float* d2);
void orc_knn_brute(const float* q, int nq, const float* t, int nt, int k, int32_t* idx, float* d2);
void orc_range_search(const float* q, int nq, const float* t, int nt, float r, int box, int maxk, int32_t* idx,
                      int32_t* cnt);

/* ---- pose */
void orc_transform_f32(const double* T16, const float* in, int n, float* out);
/* Least-squares rigid transform q ~ R p + t over pairs (FP64, Horn's
 * quaternion method; same minimiser as Umeyama's SVD form). Returns 0 if n<3. */
int orc_rigid_fit(const float* p, const float* q, const int32_t* corr, int n, double* T16);

/* ---- ICP (function.h:111-148 keyPointICP → PCL IterativeClosestPoint) */
typedef struct orc_icp_out {
  double pose[16];
  double fitness;
  int iterations;
  int converged;
  int n_corr;
} orc_icp_out;
/* A target grid kept across calls: exact 1-NN, inlier fractions of posed
 * source subsets, and ICP against it (results equal the one-shot calls'). */
typedef struct orc_grid orc_grid;
orc_grid* orc_grid_create(const float* pts, int n, float cell);
void orc_grid_destroy(orc_grid* g);
void orc_grid_nn1(const orc_grid* g, const float* q, int nq, float r2max, int32_t* idx, float* d2);
void orc_grid_inlier_fraction(const orc_grid* g, const float* src, int ns, int stride, const double* poses16,
                              int nh, float r, double* scores);
void orc_grid_icp(const orc_grid* g, const float* src, int ns, int max_it, float max_dist, double eps_t,
                  double eps_r, const double* init16, orc_icp_out* out);
void orc_grid_icp_multi(const orc_grid* g, const float* src, int ns, int max_it, float max_dist,
                        const double* inits16, int nh, orc_icp_out* outs);
/* Full oracle ICP: fixed max_iterations unless eps_t > 0 criteria stop it. */
void orc_icp(const float* src, int ns, const float* tgt, int nt, int max_it, float max_dist,
             double eps_t, double eps_r, const double* init16, orc_icp_out* out,
             double* trace_pose, int32_t* trace_corr);
/* Replay: for each iteration k, transform the source with the GIVEN pose
 * poses_in[k] (rounded to float like the GPU), find exact correspondences
 * (corr_out[k]), fit in FP64 and write poses_out[k+1] = dT * poses_in[k]. */
void orc_icp_replay(const float* src, int ns, const float* tgt, int nt, float max_dist,
                    const double* poses_in, int iters, int32_t* corr_out, double* poses_out,
                    int32_t* ncorr_out);

/* ---- TDF (kernel.cu:8-31): out[v] = min(900, min_i |v - occ_i|^2) */
void orc_tdf(const int32_t* occ, int n_occ, int dim, float* out);

/* ---- voxel-grid downsample (PCL VoxelGrid, implicit in the reference's
 * octree voxel centres, key_point.h:143-160, 287-293).  Voxel of p:
 * floor(p * (1/leaf)) per axis in FP32; output voxels in ascending linear key
 * (x fastest, relative to the minimum voxel); centroid = FP32 sum of the
 * voxel's points in ascending input index, divided by the count.  Returns V
 * (or -1 when the key space exceeds 2^32). */
int orc_voxel_downsample(const float* pts, int n, float leaf, float* out);

/* ---- normals (PCL NormalEstimation, k nearest incl. the point itself):
 * mean of the k neighbours (FP32, kNN order), covariance of the centred
 * neighbours, Jacobi eigen-solve (orc_eig3), normal = eigenvector of the
 * smallest eigenvalue flipped towards vp, curvature = l_min / (l0+l1+l2).
 * out: [n][4] = (nx, ny, nz, curvature). */
void orc_normals(const float* pts, int n, int k, const float* vp3, float* out);
/* Symmetric 3x3 eigen-decomposition, FP32 cyclic Jacobi with a fixed rule
 * set shared with the GPU; eigenvalues ascending, vectors in columns. */
void orc_eig3(const float* A9, float* w3, float* V9);

/* ---- uniform sampling (PCL UniformSampling): per voxel of edge r (voxel
 * floor(p / r)), keep the point nearest the voxel centre (ties: lowest
 * index); indices in ascending voxel key.  Returns K. */
int orc_uniform_sample(const float* pts, int n, float r, int32_t* out_idx);

/* ---- SHOT-style 352-d descriptor (Tombari, Salti, Di Stefano 2010) with the
 * conventions in oracle.c.  keys: indices into pts. */
void orc_set_shot_flags(int flags);
/* the atan2 of the SHOT angle bins (the GPU kernel runs the same operations) */
float orc_shot_atan2(float y, float x);
void orc_shot352(const float* pts, const float* normals, int n, const int32_t* keys, int nk,
                 float radius, float* desc, float* lrf9);

/* ---- descriptor 1-NN (FP32, sequential sum over the 352 dims). */
void orc_match(const float* q, int nq, const float* db, int ndb, int dim, int32_t* idx, float* d2);

/* ---- outward normals of a full model cloud (orient.c) */
void orc_orient_outward(const float* pts, float* nrm, int n, float rc, float gap, float len);

/* ---- geometric-consistency grouping (Chen & Bhanu 2007 / PCL GC) */
int orc_gc_group(const float* model_kp, const float* scene_kp, const int32_t* corr_m,
                 const int32_t* corr_s, const float* corr_d, int nc, float gc_size, int gc_thresh,
                 int max_clusters, int32_t* cluster_of, double* poses16, int32_t* sizes);

/* ---- the reference's own descriptor route (refmatch.c) */
long long orc_ref_occupancy(const float* cloud, int n, const float* keys, int nk, float res, float half,
                            int32_t* number, int32_t* offsets, int32_t* indices, long long cap);
int orc_ref_tdf(const float* cloud, const float* keys, int nk, const int32_t* offsets, const int32_t* indices,
                float res, float half, float* tdf);
void orc_ref_distance(const float* mcloud, const float* mkeys, const int32_t* moff, const int32_t* midx,
                      const float* mtdf, int nm, const float* skeys, int ns, const int32_t* pair_m,
                      const int32_t* pair_s, long long np, float res, float half, int float_order, float* score,
                      float* T);
int orc_ref_gates(const float* km, int nm_number, const double* mv3, const float* ks, int ns_number,
                  const double* sv3);
long long orc_ref_correspond(const float* mkeys, const int32_t* mnum, const double* mv3, int nm, const float* skeys,
                             const int32_t* snum, const double* sv3, int ns, const float* score_all,
                             float max_score, int32_t* pair_idx, long long cap);
int orc_ref_ransac(const float* mkeys, const float* skeys, int ns, const int32_t* pair_idx, int np,
                   const float* score_all, const float* T_all, float inlier, float max_des, float* T_out,
                   int32_t* best_inliers);

/* ---- plane segmentation + plane-area vector (planes.c) ---- */
typedef struct {
  double area;      /* 2-D convex hull area of the inliers in the plane   */
  double perimeter; /* that hull's perimeter                              */
  float coeffs[4];  /* unit normal (a, b, c) and d                         */
  int is_vertical;  /* 0 horizontal, 1 vertical, -1 neither               */
  int kept;         /* horizontal or vertical with area >= min_area        */
  int n_inliers;
  int hull_vertices;
  int flat;         /* smallest / largest inlier covariance eigenvalue < 1e-3 */
  int pad;
} orc_surface;
void orc_plane_basis(const float* c, float* e1, float* e2);
void orc_hull_measure(const void* hull_uv, int h, double* area, double* perim);
int orc_plane_class(const float* c);
int orc_plane_segment(const float* pts, int n, int max_iterations, float distance, double remain_frac,
                      double min_area, uint64_t seed, int max_planes, orc_surface* out, int* n_total);
void orc_vector3d(const float* keys, int nk, const orc_surface* s, int ns, double* v3);

/* ---- Harris3D keypoints (harris.c): keys [K][4] = x, y, z, response;
 * src[K] = the keypoint's point index (optional); returns K ---- */
int orc_harris3d(const float* pts, int n, float r, float thr, int non_max, int refine, float* keys, int32_t* src);

#ifdef __cplusplus
}
#endif
#endif

// realtime_robot_demo.cpp — main (RealTimeRobot.cpp:30-110) on the C++
// entry points of realtime_robot.hpp, with seeded synthetic clouds in place
// of the PCD files: the box chair as the model (chair1.pcd's role) and a
// cropped, moved, noisy copy of it as the scan (T0_m8111.pcd's role).
//
// Flow as in main: ModelPoint / ScanPoint keypoints and descriptors, the
// correspondence loop, Ransac (grouping, verification against the scan, ICP
// refinement of the best candidates), the scan moved onto the model,
// then keyPointICP refines model onto scan.  Prints the pair count, both
// poses and their error against the generator's transform; exits 0 when the
// refined pose is within 1 cm / 1 degree of it, 1 otherwise, 2 on an error.
// `realtime_robot_demo ref <seed>` runs main's own descriptor route instead
// (occupancy grids, TDF, get_Distance, the gates) on the kept KeyPoint calls;
// `realtime_robot_demo pcd <in> <ascii out> <binary out>` round-trips a PCD
// file through pcl::io (no GPU).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "realtime_robot.hpp"

using rtr_robot::Cloud;

static Cloud::Ptr to_cloud(const std::vector<float>& xyz4, int n) {
  Cloud::Ptr c(new Cloud);
  c->points.resize((size_t)n);
  for (int i = 0; i < n; ++i) c->points[(size_t)i] = pcl::PointXYZ(xyz4[4 * i], xyz4[4 * i + 1], xyz4[4 * i + 2]);
  c->width = (uint32_t)n;
  return c;
}

// translation (m) and rotation (rad) between two model->scene poses
static void pose_error(const Eigen::Matrix4f& A, const double* B, double* dt, double* dr) {
  double t2 = 0.0, tr = 0.0;
  for (int r = 0; r < 3; ++r) {
    const double d = A(r, 3) - B[r * 4 + 3];
    t2 += d * d;
    for (int c = 0; c < 3; ++c) tr += (double)A(r, c) * B[r * 4 + c];  // trace(A_R^T B_R)
  }
  *dt = std::sqrt(t2);
  *dr = std::acos(std::fmax(-1.0, std::fmin(1.0, 0.5 * (tr - 1.0))));
}

// main's own descriptor route (RealTimeRobot.cpp:56-102) on the kept
// KeyPoint members, one keypoint and one pair per call as main makes them:
// a 3,000-point chair and a second sampling of it moved by (dx, 0, 0), every
// 150th / 200th point a keypoint.  Prints every pair as
// "pair m s <score bits in hex> <kept>" and the count of kept pairs.
static int reference_route(unsigned long long seed) {
  const int n = 3000;
  std::vector<float> model(4 * (size_t)n), scan(4 * (size_t)n);
  rtr_robot::check(rtr_synth_shape(0, 40 + seed, n, model.data()), "rtr_synth_shape");
  rtr_robot::check(rtr_synth_shape(0, 41 + seed, n, scan.data()), "rtr_synth_shape");
  for (int i = 0; i < n; ++i) scan[4 * (size_t)i] += 0.01f * (float)(seed % 5);
  Cloud::Ptr mcloud = to_cloud(model, n), cloud = to_cloud(scan, n);
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  // main's plane areas (model_point.h:170-245, scan_point.h:117-188), which
  // fill each keypoint's vector3D for the area gate
  rtr_robot::ModelPoint modelpoint(mcloud);
  modelpoint.getArea(mcloud);
  rtr_robot::ScanPoint scanpoint(cloud);
  scanpoint.get_Area(cloud);
  std::vector<rtr_robot::KeyPoint> mk, sk;
  for (int i = 0; i < n; i += 150) {
    rtr_robot::KeyPoint p(mcloud->points[(size_t)i]);
    p.getOccupiedGrid(mcloud);
    p.get_TSDF(mcloud);
    p.get_Vector3D(modelpoint.surface);
    mk.push_back(std::move(p));
  }
  for (int i = 0; i < n; i += 200) {
    rtr_robot::KeyPoint p(cloud->points[(size_t)i]);
    p.getOccupiedGrid(cloud);
    p.get_Vector3D(scanpoint.surface);
    sk.push_back(std::move(p));
  }
  const auto t1 = clk::now();
  std::printf("surfaces %zu %zu\n", modelpoint.surface.size(), scanpoint.surface.size());
  // the reference's detector on the same clouds (its keypoints are where
  // main runs this route; the fixed strides above keep the pair count even)
  std::printf("harris %zu %zu\n", rtr_robot::harris_keypoints(*mcloud).size(), rtr_robot::harris_keypoints(*cloud).size());
  int kept = 0;
  const auto t2 = clk::now();
  for (size_t m = 0; m < mk.size(); ++m)
    for (size_t s = 0; s < sk.size(); ++s) {
      Eigen::Matrix4f T;
      const float d = rtr_robot::get_Distance(T, mk[m], sk[s]);
      const bool keydistance = d < 3;
      const bool keep = rtr_robot::match_by_height(mk[m].Key_coordinate, sk[s].Key_coordinate) &&
                        rtr_robot::match_by_area(mk[m].vector3D, sk[s].vector3D) &&
                        rtr_robot::match_by_occupied(mk[m].Occupiedgrid, sk[s].Occupiedgrid) && keydistance;
      uint32_t bits;
      std::memcpy(&bits, &d, 4);
      std::printf("pair %zu %zu %08x %d\n", m, s, bits, keep ? 1 : 0);
      kept += keep;
    }
  const auto t3 = clk::now();
  std::printf("reference route: %zu x %zu keypoints, %d pairs\n", mk.size(), sk.size(), kept);
  // wall clock of main's route through the kept API: surfaces and keypoint
  // members (getArea / get_Area, getOccupiedGrid, get_TSDF, get_Vector3D),
  // then the pair loop (get_Distance and the gates, printing included)
  const double s_keys = std::chrono::duration<double>(t1 - t0).count();
  const double s_pairs = std::chrono::duration<double>(t3 - t2).count();
  std::printf("timing keypoints %zu keypoint_s %.6f pairs %zu pair_s %.6f\n", mk.size() + sk.size(), s_keys,
              mk.size() * sk.size(), s_pairs);
  return 0;
}

int main(int argc, char** argv) {
  if (argc > 1 && std::string(argv[1]) == "pcd") {
    // pcd <in> <out ascii> <out binary>: pcl::io round trip (no GPU)
    if (argc != 5) return 2;
    Cloud c;
    if (pcl::io::loadPCDFile(argv[2], c) != 0) {
      std::fprintf(stderr, "error: cannot read %s\n", argv[2]);
      return 2;
    }
    if (pcl::io::savePCDFileASCII(argv[3], c) != 0 || pcl::io::savePCDFileBinary(argv[4], c) != 0) return 2;
    std::printf("points %zu\n", c.size());
    return 0;
  }
  if (argc > 1 && std::string(argv[1]) == "ref") {
    try {
      return reference_route(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 0ull);
    } catch (const std::exception& e) {
      std::fprintf(stderr, "error: %s\n", e.what());
      return 2;
    }
  }
  const unsigned long long seed = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 0ull;
  try {
    // the clouds (main loads chair1.pcd and T0_m8111.pcd)
    const int n = 20000;
    std::vector<float> model(4 * (size_t)n), part(4 * (size_t)n), scan(4 * (size_t)n);
    rtr_robot::check(rtr_synth_shape(0, 2024, n, model.data()), "rtr_synth_shape");
    rtr_robot::check(rtr_synth_shape(0, 500 + seed, n, part.data()), "rtr_synth_shape");
    const int kept = rtr_synth_crop(part.data(), n, 0.4, seed, scan.data());
    double T[16];
    rtr_synth_rigid(100 + seed, 30.0, 0.3, T);
    rtr_synth_transform_noise(scan.data(), kept, T, 0.002, 9 + seed, scan.data());
    Cloud::Ptr mcloud = to_cloud(model, n), cloud = to_cloud(scan, kept);

    rtr_robot::ModelPoint modelpoint(mcloud);
    modelpoint.getKeypoint();
    rtr_robot::ScanPoint scanpoint(cloud);
    scanpoint.orient_outward = true;  // a segmented object, not one sensor view
    scanpoint.getKeypoint();
    std::vector<rtr_robot::PairPoint> pairpoint = rtr_robot::match_keypoints(modelpoint, scanpoint);
    std::cout << "model keypoints " << modelpoint.n_kp << ", scan keypoints " << scanpoint.n_kp << ", pairs "
              << pairpoint.size() << std::endl;

    // Ransac gives scan -> model; main moves the scan with it
    const Eigen::Matrix4f to_model = rtr_robot::Ransac(pairpoint, 20, cloud, mcloud);
    Cloud::Ptr moved(new Cloud);
    pcl::transformPointCloud(*cloud, *moved, to_model);
    // keyPointICP refines model onto the (original) scan, starting from the
    // grouping's pose inverted back to model -> scene
    Eigen::Matrix4f init = Eigen::Matrix4f::Identity();
    for (int r = 0; r < 3; ++r) {
      float t = 0.f;
      for (int c = 0; c < 3; ++c) {
        init(r, c) = to_model(c, r);
        t -= to_model(c, r) * to_model(c, 3);
      }
      init(r, 3) = t;
    }
    const Eigen::Matrix4f refined = rtr_robot::keyPointICP_pose(nullptr, nullptr, cloud, mcloud, &init, 30, 0.02f);
    std::cout << refined;
    double dt0, dr0, dt1, dr1;
    pose_error(init, T, &dt0, &dr0);
    pose_error(refined, T, &dt1, &dr1);
    std::printf("grouping pose error %.4f m %.4f deg; refined %.4f m %.4f deg\n", dt0, dr0 * 57.29577951308232,
                dt1, dr1 * 57.29577951308232);
    return (dt1 < 0.01 && dr1 < 0.017453292519943295) ? 0 : 1;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 2;
  }
}

// realtime_robot.hpp — the reference's C++ entry points for the registration
// path, kept by name and argument meaning, on top of the rtr C ABI (rtr.h):
//
//   ModelPoint(Ptr) / getKeypoint()      model_point.h:82-94, 99-156
//   ScanPoint(Ptr)  / getKeypoint()      scan_point.h:50-53, 57-113
//   KeyPoint, PairPoint                  key_point.h:59-86, matching.h
//   the all-pairs correspondence loop    RealTimeRobot.cpp:70-102  -> match_keypoints()
//   Eigen::Matrix4f Ransac(...)          function.h:35-109
//   void keyPointICP(...)                function.h:111-148
//   ComputeTDFWithCuda                   kernel.cu:34-106 (declared in rtr.h, same signature)
//
// The stages are the ones the GPU path implements: 1 cm voxels, k = 10
// normals, 2 cm uniform keypoints and SHOT-352 descriptors at 4 cm in place
// of Harris3D keypoints and TDF / plane-area descriptors; descriptor 1-NN in
// place of get_Distance and the ratio gates; geometric-consistency grouping
// in place of the pair-consensus loop; point-to-point ICP as before.  Errors
// raise rtr_error (what() carries rtr_last_error()).
//
// Without PCL and Eigen (this machine has neither) a minimal stand-in of the
// types the signatures use is defined here: pcl::PointXYZ (16 bytes, the
// layout every rtr entry point reads), pcl::PointCloud<T>, Eigen::Matrix4f,
// pcl::transformPointCloud.  Define RTR_HAVE_PCL to use the real ones.
#pragma once

#include <cuda_runtime_api.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iostream>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "rtr.h"

#ifndef RTR_HAVE_PCL
namespace Eigen {
struct Matrix4f {
  float m[16];
  Matrix4f() { std::memset(m, 0, sizeof(m)); }
  static Matrix4f Identity() {
    Matrix4f r;
    for (int i = 0; i < 4; ++i) r.m[i * 5] = 1.f;
    return r;
  }
  float& operator()(int r, int c) { return m[r * 4 + c]; }
  float operator()(int r, int c) const { return m[r * 4 + c]; }
};
inline std::ostream& operator<<(std::ostream& o, const Matrix4f& T) {
  for (int r = 0; r < 4; ++r) {
    for (int c = 0; c < 4; ++c) o << (c ? " " : "") << T(r, c);
    o << "\n";
  }
  return o;
}
}  // namespace Eigen

namespace pcl {
struct PointXYZ {
  float x = 0.f, y = 0.f, z = 0.f, pad = 1.f;
  PointXYZ() = default;
  PointXYZ(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
};
static_assert(sizeof(PointXYZ) == 16, "the rtr entry points read 16-byte points");

// pcl::ModelCoefficients: a plane's a, b, c, d in `values`.
struct ModelCoefficients {
  std::vector<float> values;
};

template <class T>
struct PointCloud {
  using Ptr = std::shared_ptr<PointCloud<T>>;
  std::vector<T> points;
  uint32_t width = 0, height = 1;
  bool is_dense = true;
  size_t size() const { return points.size(); }
  void push_back(const T& p) {
    points.push_back(p);
    width = (uint32_t)points.size();
  }
  typename std::vector<T>::iterator begin() { return points.begin(); }
  typename std::vector<T>::iterator end() { return points.end(); }
  typename std::vector<T>::const_iterator begin() const { return points.begin(); }
  typename std::vector<T>::const_iterator end() const { return points.end(); }
};

inline void transformPointCloud(const PointCloud<PointXYZ>& in, PointCloud<PointXYZ>& out,
                                const Eigen::Matrix4f& T) {
  std::vector<PointXYZ> r(in.points.size());
  for (size_t i = 0; i < r.size(); ++i) {
    const PointXYZ& p = in.points[i];
    r[i] = PointXYZ(T(0, 0) * p.x + T(0, 1) * p.y + T(0, 2) * p.z + T(0, 3),
                    T(1, 0) * p.x + T(1, 1) * p.y + T(1, 2) * p.z + T(1, 3),
                    T(2, 0) * p.x + T(2, 1) * p.y + T(2, 2) * p.z + T(2, 3));
  }
  out.points.swap(r);
  out.width = (uint32_t)out.points.size();
  out.height = 1;
}

// PCD files (pcl::io::loadPCDFile / savePCDFileASCII / savePCDFileBinary,
// as main uses them at RealTimeRobot.cpp:34-35, 108-109).  Reads PCD v0.5-0.7
// headers with DATA ascii or binary (binary_compressed is refused), takes x,
// y and z from any field layout (F 4/8, I or U 1/2/4/8 bytes, any COUNT), and
// ignores the other fields.  Writes x y z as float: ascii with 9 significant
// digits (float values read back exactly), binary as 12-byte records.
// Returns 0, or -1 on a missing file or a header / data it cannot read.
namespace io {
namespace detail {
struct PcdField {
  std::string name;
  int size = 4, count = 1;
  char type = 'F';
};

inline bool pcd_value(const unsigned char* p, const PcdField& f, double* out) {
  switch (f.type) {
    case 'F':
      if (f.size == 4) { float v; std::memcpy(&v, p, 4); *out = v; return true; }
      if (f.size == 8) { double v; std::memcpy(&v, p, 8); *out = v; return true; }
      return false;
    case 'I':
      if (f.size == 1) { int8_t v; std::memcpy(&v, p, 1); *out = v; return true; }
      if (f.size == 2) { int16_t v; std::memcpy(&v, p, 2); *out = v; return true; }
      if (f.size == 4) { int32_t v; std::memcpy(&v, p, 4); *out = v; return true; }
      if (f.size == 8) { int64_t v; std::memcpy(&v, p, 8); *out = (double)v; return true; }
      return false;
    case 'U':
      if (f.size == 1) { uint8_t v; std::memcpy(&v, p, 1); *out = v; return true; }
      if (f.size == 2) { uint16_t v; std::memcpy(&v, p, 2); *out = v; return true; }
      if (f.size == 4) { uint32_t v; std::memcpy(&v, p, 4); *out = v; return true; }
      if (f.size == 8) { uint64_t v; std::memcpy(&v, p, 8); *out = (double)v; return true; }
      return false;
  }
  return false;
}
}  // namespace detail

inline int loadPCDFile(const std::string& path, PointCloud<PointXYZ>& cloud) {
  FILE* fp = std::fopen(path.c_str(), "rb");
  if (!fp) return -1;
  std::vector<unsigned char> raw;
  unsigned char buf[65536];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof(buf), fp)) > 0) raw.insert(raw.end(), buf, buf + got);
  std::fclose(fp);
  std::vector<detail::PcdField> fields;
  long long points = -1, width = -1, height = 1;
  std::string data;
  size_t pos = 0;
  while (pos < raw.size() && data.empty()) {
    size_t end = pos;
    while (end < raw.size() && raw[end] != '\n') ++end;
    std::string line(raw.begin() + (long)pos, raw.begin() + (long)end);
    pos = end + 1;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.empty() || line[0] == '#') continue;
    std::vector<std::string> tok;
    for (size_t i = 0; i < line.size();) {
      while (i < line.size() && (line[i] == ' ' || line[i] == '\t')) ++i;
      size_t j = i;
      while (j < line.size() && line[j] != ' ' && line[j] != '\t') ++j;
      if (j > i) tok.push_back(line.substr(i, j - i));
      i = j;
    }
    if (tok.empty()) continue;
    const std::string& key = tok[0];
    if (key == "FIELDS" || key == "COLUMNS") {
      fields.assign(tok.size() - 1, detail::PcdField());
      for (size_t i = 1; i < tok.size(); ++i) fields[i - 1].name = tok[i];
    } else if (key == "SIZE" || key == "TYPE" || key == "COUNT") {
      if (tok.size() - 1 != fields.size()) return -1;
      for (size_t i = 1; i < tok.size(); ++i) {
        if (key == "SIZE") fields[i - 1].size = std::atoi(tok[i].c_str());
        if (key == "TYPE") fields[i - 1].type = tok[i][0];
        if (key == "COUNT") fields[i - 1].count = std::atoi(tok[i].c_str());
      }
    } else if (key == "WIDTH" && tok.size() > 1) {
      width = std::atoll(tok[1].c_str());
    } else if (key == "HEIGHT" && tok.size() > 1) {
      height = std::atoll(tok[1].c_str());
    } else if (key == "POINTS" && tok.size() > 1) {
      points = std::atoll(tok[1].c_str());
    } else if (key == "DATA" && tok.size() > 1) {
      data = tok[1];
    }
  }
  if (points < 0) points = width * height;
  if (points < 0 || data.empty() || fields.empty()) return -1;
  int col[3] = {-1, -1, -1};
  size_t rec = 0;
  std::vector<size_t> off(fields.size()), first_col(fields.size());
  size_t ncol = 0;
  for (size_t i = 0; i < fields.size(); ++i) {
    if (fields[i].size <= 0 || fields[i].count <= 0) return -1;
    off[i] = rec;
    first_col[i] = ncol;
    rec += (size_t)fields[i].size * (size_t)fields[i].count;
    ncol += (size_t)fields[i].count;
    for (int a = 0; a < 3; ++a)
      if (fields[i].name == std::string(1, "xyz"[a])) col[a] = (int)i;
  }
  if (col[0] < 0 || col[1] < 0 || col[2] < 0) return -1;
  if (data != "binary" && data != "ascii") return -1;  // binary_compressed (LZF) is not read
  // the data section must hold the declared points before anything is sized
  // from the header (a corrupt POINTS must not allocate): a binary record is
  // rec bytes, an ascii one at least a digit and a separator per value
  const size_t avail = pos <= raw.size() ? raw.size() - pos : 0;
  if (data == "binary" ? (size_t)points > avail / rec : (size_t)points > (avail + 1) / (2 * ncol)) return -1;
  cloud.points.assign((size_t)points, PointXYZ());
  if (data == "binary") {
    for (long long i = 0; i < points; ++i) {
      const unsigned char* r = raw.data() + pos + rec * (size_t)i;
      double v[3];
      for (int a = 0; a < 3; ++a)
        if (!detail::pcd_value(r + off[(size_t)col[a]], fields[(size_t)col[a]], &v[a])) return -1;
      cloud.points[(size_t)i] = PointXYZ((float)v[0], (float)v[1], (float)v[2]);
    }
  } else {
    std::vector<double> row(ncol);
    const char* c = reinterpret_cast<const char*>(raw.data()) + pos;
    const char* e = reinterpret_cast<const char*>(raw.data()) + raw.size();
    for (long long i = 0; i < points; ++i) {
      for (size_t k = 0; k < ncol; ++k) {
        while (c < e && (*c == ' ' || *c == '\t' || *c == '\n' || *c == '\r')) ++c;
        if (c >= e) return -1;
        std::string tokv;
        while (c < e && *c != ' ' && *c != '\t' && *c != '\n' && *c != '\r') tokv.push_back(*c++);
        row[k] = std::strtod(tokv.c_str(), nullptr);
      }
      cloud.points[(size_t)i] = PointXYZ((float)row[first_col[(size_t)col[0]]], (float)row[first_col[(size_t)col[1]]],
                                         (float)row[first_col[(size_t)col[2]]]);
    }
  }
  cloud.width = (uint32_t)points;
  cloud.height = 1;
  return 0;
}

inline int pcd_write(const std::string& path, const PointCloud<PointXYZ>& cloud, bool binary) {
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) return -1;
  const size_t n = cloud.points.size();
  std::fprintf(fp,
               "# .PCD v0.7 - Point Cloud Data file format\nVERSION 0.7\nFIELDS x y z\nSIZE 4 4 4\nTYPE F F F\n"
               "COUNT 1 1 1\nWIDTH %zu\nHEIGHT 1\nVIEWPOINT 0 0 0 1 0 0 0\nPOINTS %zu\nDATA %s\n",
               n, n, binary ? "binary" : "ascii");
  for (size_t i = 0; i < n; ++i) {
    const PointXYZ& p = cloud.points[i];
    if (binary) {
      const float v[3] = {p.x, p.y, p.z};
      std::fwrite(v, sizeof(float), 3, fp);
    } else {
      std::fprintf(fp, "%.9g %.9g %.9g\n", (double)p.x, (double)p.y, (double)p.z);
    }
  }
  return std::fclose(fp) == 0 ? 0 : -1;
}

inline int savePCDFileASCII(const std::string& path, const PointCloud<PointXYZ>& cloud) {
  return pcd_write(path, cloud, false);
}
inline int savePCDFileBinary(const std::string& path, const PointCloud<PointXYZ>& cloud) {
  return pcd_write(path, cloud, true);
}
}  // namespace io
}  // namespace pcl
#endif  // RTR_HAVE_PCL

namespace rtr_robot {

using Cloud = pcl::PointCloud<pcl::PointXYZ>;

struct rtr_error : std::runtime_error {
  rtr_status status;
  rtr_error(rtr_status s, const std::string& where)
      : std::runtime_error(where + ": " + rtr_status_string(s) + ": " + rtr_last_error()), status(s) {}
};

inline void check(rtr_status s, const char* where) {
  if (s != RTR_OK) throw rtr_error(s, where);
}

inline void check_cuda(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(where) + ": " + cudaGetErrorString(e));
}

// Device buffer owned by the host objects below.
template <class T>
struct DeviceArray {
  T* p = nullptr;
  size_t n = 0;
  DeviceArray() = default;
  explicit DeviceArray(size_t count) { resize(count); }
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  DeviceArray(DeviceArray&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr, o.n = 0; }
  ~DeviceArray() { cudaFree(p); }
  void resize(size_t count) {
    cudaFree(p);
    p = nullptr;
    n = count;
    if (count) check_cuda(cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T)), "cudaMalloc");
  }
  void upload(const T* h, size_t count) {
    if (count > n) resize(count);
    if (count) check_cuda(cudaMemcpy(p, h, count * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
  }
  void download(T* h, size_t count) const {
    if (count) check_cuda(cudaMemcpy(h, p, count * sizeof(T), cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
  }
};

// One context per host thread (the reference is single-threaded; so is the
// context).
inline rtr_context* thread_context() {
  struct Holder {
    rtr_context* ctx = nullptr;
    ~Holder() {
      if (ctx) rtr_context_destroy(ctx);
    }
  };
  thread_local Holder h;
  if (!h.ctx) check(rtr_context_create(0, &h.ctx), "rtr_context_create");
  return h.ctx;
}

// Device scratch of the calling thread for the temporaries of one call: a
// single buffer that only grows (a cudaMalloc only when a call needs more
// than any before it), carved per call.  A call lists its arrays, commits,
// then uses them; calls do not nest (each finishes with a synchronous copy
// back, so the next call may reuse the bytes).
struct ThreadArena {
  char* base = nullptr;
  size_t cap = 0;
  ~ThreadArena() { cudaFree(base); }
};
inline ThreadArena& thread_arena() {
  thread_local ThreadArena a;
  return a;
}
class Carve {
 public:
  template <class T>
  Carve& add(T*& out, size_t count) {
    const size_t o = off_;
    set_.push_back([&out, o](char* b) { out = reinterpret_cast<T*>(b + o); });
    off_ += (count * sizeof(T) + 255) & ~size_t(255);
    return *this;
  }
  void commit() {
    ThreadArena& a = thread_arena();
    if (off_ > a.cap) {
      const size_t want = off_ > 2 * a.cap ? off_ : 2 * a.cap;
      cudaFree(a.base);
      a.base = nullptr;
      a.cap = 0;
      check_cuda(cudaMalloc(reinterpret_cast<void**>(&a.base), want), "cudaMalloc");
      a.cap = want;
    }
    for (auto& f : set_) f(a.base);
  }

 private:
  std::vector<std::function<void(char*)>> set_;
  size_t off_ = 0;
};
template <class T>
inline void to_device(T* d, const T* h, size_t count) {
  if (count) check_cuda(cudaMemcpy(d, h, count * sizeof(T), cudaMemcpyHostToDevice), "cudaMemcpy H2D");
}
template <class T>
inline void to_host(T* h, const T* d, size_t count) {
  if (count) check_cuda(cudaMemcpy(h, d, count * sizeof(T), cudaMemcpyDeviceToHost), "cudaMemcpy D2H");
}

constexpr int kDescDim = 352;

// Surface (key_point.h:47-51): one plane of the reference's surface list.
struct Surface {
  double Area = 0.0;
  pcl::ModelCoefficients Coefficients;
  bool IsVertical = false;
};

// getArea / get_Area (model_point.h:170-245, scan_point.h:117-188) through
// rtr_plane_segment: the kept planes (horizontal or vertical, area >= 0.16)
// in extraction order.  The plane's area is its inliers' 2-D convex-hull
// area in the plane.
inline std::vector<Surface> segment_surfaces(const Cloud& cloud, std::vector<rtr_surface>* all = nullptr) {
  rtr_context* ctx = thread_context();
  const int n = (int)cloud.size();
  std::vector<Surface> out;
  if (n == 0) return out;
  float* d_pts;
  Carve().add(d_pts, 4 * (size_t)n).commit();
  to_device(d_pts, reinterpret_cast<const float*>(cloud.points.data()), 4 * (size_t)n);
  rtr_plane_params prm;
  rtr_plane_default_params(&prm);
  std::vector<rtr_surface> s(256);
  int ns = 0;
  check(rtr_plane_segment(ctx, d_pts, n, &prm, s.data(), (int)s.size(), &ns, nullptr), "rtr_plane_segment");
  s.resize((size_t)ns);
  for (const rtr_surface& r : s) {
    if (!r.kept) continue;
    Surface t;
    t.Area = r.area;
    t.Coefficients.values.assign(r.coeffs, r.coeffs + 4);
    t.IsVertical = r.is_vertical == 1;
    out.push_back(t);
  }
  if (all) *all = s;
  return out;
}

// The kept surfaces back in the C ABI's record form (for rtr_vector3d).
inline std::vector<rtr_surface> to_records(const std::vector<Surface>& surface) {
  std::vector<rtr_surface> r(surface.size());
  for (size_t i = 0; i < surface.size(); ++i) {
    std::memset(&r[i], 0, sizeof(rtr_surface));
    r[i].area = surface[i].Area;
    for (int k = 0; k < 4; ++k)
      r[i].coeffs[k] = k < (int)surface[i].Coefficients.values.size() ? surface[i].Coefficients.values[(size_t)k] : 0.f;
    r[i].is_vertical = surface[i].IsVertical ? 1 : 0;
    r[i].kept = 1;
  }
  return r;
}

// OccupiedGrid (key_point.h:52-57): the points of the keypoint's box and the
// number of occupied 1 cm leaves among them.
struct OccupiedGrid {
  Cloud::Ptr cloud{new Cloud};
  float Border[6] = {0, 0, 0, 0, 0, 0};
  int Number = 0;
};

// A keypoint (key_point.h:59-86).  The SHOT route fills `descriptor`; the
// reference's own route fills Occupiedgrid (getOccupiedGrid), grid_value and
// Border (get_TSDF); vector3D is the plane-area vector (0.16 each as the
// reference's constructor sets it, until get_Vector3D over the cloud's
// surfaces fills it).
struct KeyPoint {
  pcl::PointXYZ Key_coordinate;
  std::vector<float> descriptor;  // kDescDim values, L2-normalised
  OccupiedGrid Occupiedgrid;
  std::vector<double> vector3D{0.16, 0.16, 0.16};
  std::vector<float> grid_value;  // 27000 values after get_TSDF
  float Border[6] = {0, 0, 0, 0, 0, 0};
  KeyPoint() = default;
  explicit KeyPoint(const pcl::PointXYZ& p) : Key_coordinate(p) {}

  // key_point.h:112-161 through rtr_ref_occupancy (one keypoint).
  void getOccupiedGrid(Cloud::Ptr cloud, float resolution = 0.01f, float f_adjust = 0.1f);
  // key_point.h:251-334 through rtr_ref_tdf, from Occupiedgrid.cloud.
  void get_TSDF(Cloud::Ptr cloud, float resolution = 0.01f, float f_adjust = 0.15f);
  // key_point.h:87-111 through rtr_vector3d (vector3d_all does many at once).
  void get_Vector3D(std::vector<Surface>& surface);
};

// get_Vector3D for many keypoints in one rtr_vector3d call.
inline void vector3d_all(std::vector<KeyPoint>& keys, const std::vector<Surface>& surface) {
  if (keys.empty()) return;
  rtr_context* ctx = thread_context();
  std::vector<float> k(4 * keys.size());
  for (size_t i = 0; i < keys.size(); ++i) {
    k[4 * i] = keys[i].Key_coordinate.x;
    k[4 * i + 1] = keys[i].Key_coordinate.y;
    k[4 * i + 2] = keys[i].Key_coordinate.z;
    k[4 * i + 3] = 0.f;
  }
  float* d_k;
  double* d_v;
  Carve().add(d_k, k.size()).add(d_v, 3 * keys.size()).commit();
  to_device(d_k, k.data(), k.size());
  const std::vector<rtr_surface> rec = to_records(surface);
  check(rtr_vector3d(ctx, d_k, (int)keys.size(), rec.data(), (int)rec.size(), d_v, nullptr), "rtr_vector3d");
  std::vector<double> v(3 * keys.size());
  to_host(v.data(), d_v, v.size());
  for (size_t i = 0; i < keys.size(); ++i) keys[i].vector3D.assign(v.begin() + 3 * i, v.begin() + 3 * i + 3);
}

inline void KeyPoint::get_Vector3D(std::vector<Surface>& surface) {
  std::vector<KeyPoint> one(1, *this);
  vector3d_all(one, surface);
  vector3D = one[0].vector3D;
}

// A model keypoint paired with a scene keypoint (point_i model, point_j
// scene, as main builds them), with the descriptor distance that ranks it.
struct PairPoint {
  KeyPoint point_i, point_j;
  int model_index = -1, scene_index = -1;
  float distance2 = 0.f;
};

// Keypoints and descriptors of a cloud: voxels, normals, uniform keypoints,
// SHOT (the body of both getKeypoint()s).  Device copies are kept for the
// matching and grouping stages.
struct KeypointSet {
  Cloud key_coordinates;
  std::vector<KeyPoint> keyPoint;
  DeviceArray<float> d_kp;    // K x 4
  DeviceArray<float> d_desc;  // K x 352
  int n_kp = 0;

  void compute(const Cloud& cloud, const float viewpoint[3], bool outward, bool model_side) {
    rtr_context* ctx = thread_context();
    rtr_recog_params prm;
    rtr_recog_default_params(&prm);
    const int n = (int)cloud.size();
    if (n <= 0) throw std::invalid_argument("getKeypoint: empty cloud");
    float *d_pts, *d_vox, *d_nrm;
    int* d_cnt;
    int32_t* d_keys;
    Carve()
        .add(d_pts, 4 * (size_t)n)
        .add(d_vox, 4 * (size_t)n)
        .add(d_nrm, 4 * (size_t)n)
        .add(d_cnt, 2)
        .add(d_keys, (size_t)n)
        .commit();
    to_device(d_pts, reinterpret_cast<const float*>(cloud.points.data()), 4 * (size_t)n);
    check(rtr_voxel_downsample(ctx, d_pts, n, prm.voxel_leaf, d_vox, d_cnt, nullptr), "rtr_voxel_downsample");
    int V = 0;
    to_host(&V, d_cnt, 1);
    if (V <= 0) throw std::runtime_error("getKeypoint: the voxel filter kept no point");
    check(rtr_normals(ctx, d_vox, V, prm.normal_k, viewpoint, 2.f * prm.voxel_leaf, d_nrm, nullptr), "rtr_normals");
    if (outward) check(rtr_orient_normals_outward(ctx, d_vox, d_nrm, V, 0.01f, 0.005f, 1.0f, nullptr),
                       "rtr_orient_normals_outward");
    const float r_kp = model_side ? prm.model_keypoint_r : prm.scene_keypoint_r;
    check(rtr_uniform_sample(ctx, d_vox, V, r_kp, d_keys, d_cnt + 1, nullptr), "rtr_uniform_sample");
    int K = 0;
    to_host(&K, d_cnt + 1, 1);
    n_kp = K;
    d_desc.resize((size_t)K * kDescDim);
    if (K > 0)
      check(rtr_shot352(ctx, d_vox, d_nrm, V, d_keys, K, prm.descriptor_r, d_desc.p, nullptr, nullptr),
            "rtr_shot352");
    std::vector<float> vox(4 * (size_t)V), desc((size_t)K * kDescDim);
    std::vector<int32_t> keys((size_t)K);
    to_host(vox.data(), d_vox, vox.size());
    to_host(keys.data(), d_keys, keys.size());
    d_desc.download(desc.data(), desc.size());
    std::vector<float> kp(4 * (size_t)K);
    key_coordinates = Cloud();
    keyPoint.assign((size_t)K, KeyPoint());
    for (int i = 0; i < K; ++i) {
      const float* v = &vox[4 * (size_t)keys[i]];
      pcl::PointXYZ p(v[0], v[1], v[2]);
      key_coordinates.push_back(p);
      keyPoint[i] = KeyPoint(p);
      keyPoint[i].descriptor.assign(desc.begin() + (size_t)i * kDescDim, desc.begin() + (size_t)(i + 1) * kDescDim);
      std::memcpy(&kp[4 * (size_t)i], v, 3 * sizeof(float));
      kp[4 * (size_t)i + 3] = 0.f;
    }
    d_kp.upload(kp.data(), kp.size());
  }
};

// The reference's own detector (model_point.h:127-136, scan_point.h:85-94:
// HarrisKeypoint3D, radius 0.05, threshold 0.01, non-maximum suppression)
// through rtr_harris3d: the keypoint positions of `cloud`.
inline Cloud harris_keypoints(const Cloud& cloud, float radius = 0.05f, float threshold = 0.01f) {
  rtr_context* ctx = thread_context();
  const int n = (int)cloud.size();
  Cloud out;
  if (n == 0) return out;
  float *d_pts, *d_keys;
  int32_t* d_src;
  int* d_cnt;
  Carve().add(d_pts, 4 * (size_t)n).add(d_keys, 4 * (size_t)n).add(d_src, (size_t)n).add(d_cnt, 1).commit();
  to_device(d_pts, reinterpret_cast<const float*>(cloud.points.data()), 4 * (size_t)n);
  rtr_harris_params prm;
  rtr_harris_default_params(&prm);
  prm.radius = radius;
  prm.threshold = threshold;
  check(rtr_harris3d(ctx, d_pts, n, &prm, d_keys, d_src, d_cnt, nullptr), "rtr_harris3d");
  int K = 0;
  to_host(&K, d_cnt, 1);
  std::vector<float> k(4 * (size_t)K);
  to_host(k.data(), d_keys, k.size());
  for (int i = 0; i < K; ++i) out.push_back(pcl::PointXYZ(k[4 * (size_t)i], k[4 * (size_t)i + 1], k[4 * (size_t)i + 2]));
  return out;
}

// model_point.h:82-94: the model cloud (a full 360-degree cloud: normals are
// oriented outward; keypoints at the model radius).
class ModelPoint : public KeypointSet {
 public:
  Cloud::Ptr Mpoint;
  std::vector<Surface> surface;
  ModelPoint() = default;
  explicit ModelPoint(Cloud::Ptr m) : Mpoint(std::move(m)) {}
  void getKeypoint() {
    const float vp[3] = {0.f, 0.f, 0.f};
    compute(*Mpoint, vp, true, true);
  }
  // model_point.h:170-245
  void getArea(Cloud::Ptr modelPoint) {
    const std::vector<Surface> s = segment_surfaces(*modelPoint);
    surface.insert(surface.end(), s.begin(), s.end());
  }
};

// scan_point.h:50-53: the scene.  A sensor view keeps its normals facing
// `viewpoint`; a segmented object seen from all sides (orient_outward) has
// them oriented outward like the model's.
class ScanPoint : public KeypointSet {
 public:
  Cloud::Ptr Spoint;
  std::vector<Surface> surface;
  // scan_point.h:117-188
  void get_Area(Cloud::Ptr scanPoint) {
    const std::vector<Surface> s = segment_surfaces(*scanPoint);
    surface.insert(surface.end(), s.begin(), s.end());
  }
  float viewpoint[3] = {0.f, 0.f, 0.f};
  bool orient_outward = false;
  ScanPoint() = default;
  explicit ScanPoint(Cloud::Ptr s) : Spoint(std::move(s)) {}
  void getKeypoint() { compute(*Spoint, viewpoint, orient_outward, false); }
};

// The correspondence loop of main (RealTimeRobot.cpp:70-102): every scene
// keypoint paired with its nearest model descriptor, kept when the squared
// descriptor distance is below max_d2 (the recognition default, 0.25).
inline std::vector<PairPoint> match_keypoints(const ModelPoint& model, const ScanPoint& scan, float max_d2 = -1.f) {
  rtr_context* ctx = thread_context();
  if (max_d2 < 0.f) {
    rtr_recog_params prm;
    rtr_recog_default_params(&prm);
    max_d2 = prm.match_max_d2;
  }
  std::vector<PairPoint> out;
  if (model.n_kp == 0 || scan.n_kp == 0) return out;
  int32_t* d_idx;
  float* d_d2;
  Carve().add(d_idx, (size_t)scan.n_kp).add(d_d2, (size_t)scan.n_kp).commit();
  check(rtr_match(ctx, scan.d_desc.p, scan.n_kp, model.d_desc.p, model.n_kp, d_idx, d_d2, nullptr), "rtr_match");
  std::vector<int32_t> idx((size_t)scan.n_kp);
  std::vector<float> d2((size_t)scan.n_kp);
  to_host(idx.data(), d_idx, idx.size());
  to_host(d2.data(), d_d2, d2.size());
  for (int s = 0; s < scan.n_kp; ++s) {
    if (idx[s] < 0 || !(d2[s] < max_d2)) continue;
    PairPoint p;
    p.point_i = model.keyPoint[(size_t)idx[s]];
    p.point_j = scan.keyPoint[(size_t)s];
    p.model_index = idx[s];
    p.scene_index = s;
    p.distance2 = d2[s];
    out.push_back(std::move(p));
  }
  return out;
}

// ---- the reference's own descriptor route, one keypoint / pair per call ----
inline void KeyPoint::getOccupiedGrid(Cloud::Ptr cloud, float resolution, float f_adjust) {
  rtr_context* ctx = thread_context();
  const int n = (int)cloud->size();
  const float key[4] = {Key_coordinate.x, Key_coordinate.y, Key_coordinate.z, 0.f};
  const size_t cap = (size_t)(n > 0 ? n : 1);
  float *d_cloud, *d_key;
  int32_t *d_num, *d_off, *d_idx;
  Carve().add(d_cloud, 4 * cap).add(d_key, 4).add(d_num, 1).add(d_off, 2).add(d_idx, cap).commit();
  to_device(d_cloud, reinterpret_cast<const float*>(cloud->points.data()), 4 * (size_t)n);
  to_device(d_key, key, 4);
  long long total = 0;
  check(rtr_ref_occupancy(ctx, d_cloud, n, d_key, 1, resolution, f_adjust, d_num, d_off, d_idx, (long long)cap, &total,
                          nullptr),
        "rtr_ref_occupancy");
  std::vector<int32_t> idx((size_t)total);
  to_host(idx.data(), d_idx, idx.size());
  to_host(&Occupiedgrid.Number, d_num, 1);
  Occupiedgrid.cloud.reset(new Cloud);
  Occupiedgrid.cloud->points.reserve(idx.size());
  for (int32_t i : idx) Occupiedgrid.cloud->points.push_back(cloud->points[(size_t)i]);
  Occupiedgrid.cloud->width = (uint32_t)idx.size();
}

inline void KeyPoint::get_TSDF(Cloud::Ptr cloud, float resolution, float f_adjust) {
  (void)cloud;  // the reference reads Occupiedgrid.cloud here too
  rtr_context* ctx = thread_context();
  const Cloud& occ = *Occupiedgrid.cloud;
  const int n = (int)occ.size();
  const float key[4] = {Key_coordinate.x, Key_coordinate.y, Key_coordinate.z, 0.f};
  std::vector<int32_t> idx((size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) idx[(size_t)i] = i;
  const int32_t off[2] = {0, n};
  float *d_cloud, *d_key, *d_tdf;
  int32_t *d_off, *d_idx;
  Carve()
      .add(d_cloud, 4 * (size_t)(n > 0 ? n : 1))
      .add(d_key, 4)
      .add(d_tdf, 27000)
      .add(d_off, 2)
      .add(d_idx, idx.size())
      .commit();
  to_device(d_cloud, reinterpret_cast<const float*>(occ.points.data()), 4 * (size_t)n);
  to_device(d_key, key, 4);
  to_device(d_off, off, 2);
  to_device(d_idx, idx.data(), idx.size());
  int dim = 0;
  check(rtr_ref_tdf(ctx, d_cloud, d_key, 1, d_off, d_idx, resolution, f_adjust, d_tdf, &dim, nullptr), "rtr_ref_tdf");
  grid_value.assign(27000, 0.f);
  to_host(grid_value.data(), d_tdf, (size_t)dim * dim * dim);
  const float k3[3] = {Key_coordinate.x, Key_coordinate.y, Key_coordinate.z};
  for (int a = 0; a < 3; ++a) {
    Border[a] = k3[a] - f_adjust;
    Border[3 + a] = k3[a] + f_adjust;
  }
}

// matching.h:122-222 through rtr_ref_distance (one pair): p1_key is the model
// keypoint after getOccupiedGrid and get_TSDF (30^3 field), p2_scan the scan
// keypoint.  Returns the score; key_transform gets the pair's transform.
inline float get_Distance(Eigen::Matrix4f& key_transform, KeyPoint& p1_key, KeyPoint& p2_scan,
                          const float resolution = 0.01f) {
  if (p1_key.grid_value.size() != 27000) throw rtr_error(RTR_ERR_INVALID_ARG, "get_Distance: call get_TSDF first");
  rtr_context* ctx = thread_context();
  const Cloud& occ = *p1_key.Occupiedgrid.cloud;
  const int n = (int)occ.size();
  const float km[4] = {p1_key.Key_coordinate.x, p1_key.Key_coordinate.y, p1_key.Key_coordinate.z, 0.f};
  const float ks[4] = {p2_scan.Key_coordinate.x, p2_scan.Key_coordinate.y, p2_scan.Key_coordinate.z, 0.f};
  std::vector<int32_t> idx((size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) idx[(size_t)i] = i;
  const int32_t off[2] = {0, n}, pm = 0, ps = 0;
  // one upload of the packed inputs: keypoints (2 x 4 floats), the field,
  // the cloud; and of the integer inputs: offsets, pair, indices
  const size_t nf = 8 + 27000 + 4 * (size_t)n, ni = 4 + idx.size();
  std::vector<float> hf(nf);
  std::memcpy(hf.data(), km, sizeof(km));
  std::memcpy(hf.data() + 4, ks, sizeof(ks));
  std::memcpy(hf.data() + 8, p1_key.grid_value.data(), 27000 * sizeof(float));
  if (n) std::memcpy(hf.data() + 8 + 27000, occ.points.data(), 4 * (size_t)n * sizeof(float));
  std::vector<int32_t> hi(ni);
  hi[0] = off[0], hi[1] = off[1], hi[2] = pm, hi[3] = ps;
  std::memcpy(hi.data() + 4, idx.data(), idx.size() * sizeof(int32_t));
  float *d_f, *d_out;
  int32_t* d_i;
  Carve().add(d_f, nf).add(d_i, ni).add(d_out, 20).commit();
  to_device(d_f, hf.data(), nf);
  to_device(d_i, hi.data(), ni);
  check(rtr_ref_distance(ctx, d_f + 8 + 27000, d_f, 1, d_i, d_i + 4, d_f + 8, d_f + 4, 1, d_i + 2, d_i + 3, 1,
                         resolution, 0.15f, d_out, d_out + 4, nullptr),
        "rtr_ref_distance");
  float o[20];
  to_host(o, d_out, 20);
  const float score = o[0];
  const float* T = o + 4;
  for (int i = 0; i < 16; ++i) key_transform(i / 4, i % 4) = T[i];
  return score;
}

// function.h:158-178, as written: float(2/3) and float(1/3) are 0, and the
// occupancy ratio is an integer quotient.
inline bool match_by_height(pcl::PointXYZ& key1, pcl::PointXYZ& key2) {
  const float ratio = key1.z / key2.z;
  return ratio >= 0.f || ratio <= 1.5f;
}
inline bool match_by_area(std::vector<double> v1, std::vector<double> v2) {
  for (int a = 0; a < 3; ++a) {
    const double r = v1[(size_t)a] / v2[(size_t)a];
    if (r > 3 || r < 0.0) return false;
  }
  return true;
}
inline bool match_by_occupied(OccupiedGrid& o1, OccupiedGrid& o2) {
  if (o2.Number == 0) return false;
  const float q = (float)(o1.Number / o2.Number);
  return !(q > 2 || q < 0.5);
}

// function.h:35-109.  The reference scores candidate transforms and keeps
// the best.  Here the candidates are the groups of geometric-consistency
// grouping (bin 1 cm, at least 5 members, the configs' parameters), each
// with its least-squares pose, verified as the library's recognition does:
// each pose scored on the device by the model points (mcloud) it brings
// within 2 * inlier_r of a scene point (cloud, rtr_pose_inliers), the 16 best
// refined together by one multi-problem ICP (rtr_icp_multi: 30 iterations,
// 2 cm, a 3 cm target grid), and the refined pose with the most model points
// within inlier_r kept (ties: the better first score).  As in main, the
// result maps the scene onto the model (main applies it to `cloud`).
// ransac_times is kept for the signature (the grouping is deterministic).
// Identity when no group reaches 5 members.
inline Eigen::Matrix4f Ransac(std::vector<PairPoint> pairpoint, int ransac_times, Cloud::Ptr cloud, Cloud::Ptr mcloud,
                              float inlier_r = 0.01f) {
  (void)ransac_times;
  rtr_context* ctx = thread_context();
  const int C = (int)pairpoint.size();
  Eigen::Matrix4f best = Eigen::Matrix4f::Identity();
  if (C == 0) return best;
  std::vector<float> mk(4 * (size_t)C), sk(4 * (size_t)C), cd((size_t)C);
  std::vector<int32_t> cm((size_t)C), cs((size_t)C);
  for (int i = 0; i < C; ++i) {
    const PairPoint& p = pairpoint[(size_t)i];
    const pcl::PointXYZ a = p.point_i.Key_coordinate, b = p.point_j.Key_coordinate;
    mk[4 * (size_t)i] = a.x, mk[4 * (size_t)i + 1] = a.y, mk[4 * (size_t)i + 2] = a.z, mk[4 * (size_t)i + 3] = 0.f;
    sk[4 * (size_t)i] = b.x, sk[4 * (size_t)i + 1] = b.y, sk[4 * (size_t)i + 2] = b.z, sk[4 * (size_t)i + 3] = 0.f;
    cm[(size_t)i] = i;
    cs[(size_t)i] = i;
    cd[(size_t)i] = p.distance2;
  }
  constexpr int kMaxClusters = 256, kMaxMembers = 128, kTop = 16;
  const int ns = (int)cloud->size(), nm = (int)mcloud->size();
  float *d_mk, *d_sk, *d_cd, *d_s, *d_m;
  int32_t *d_cm, *d_cs, *d_mem, *d_sizes, *d_cnt;
  double *d_poses, *d_init;
  rtr_icp_result* d_res;
  Carve()
      .add(d_mk, mk.size())
      .add(d_sk, sk.size())
      .add(d_cd, cd.size())
      .add(d_cm, cm.size())
      .add(d_cs, cs.size())
      .add(d_mem, (size_t)kMaxClusters * kMaxMembers)
      .add(d_sizes, kMaxClusters)
      .add(d_poses, (size_t)kMaxClusters * 16)
      .add(d_s, 4 * (size_t)(ns > 0 ? ns : 1))
      .add(d_m, 4 * (size_t)(nm > 0 ? nm : 1))
      .add(d_cnt, kMaxClusters)
      .add(d_init, (size_t)kTop * 16)
      .add(d_res, kTop)
      .commit();
  to_device(d_mk, mk.data(), mk.size());
  to_device(d_sk, sk.data(), sk.size());
  to_device(d_cd, cd.data(), cd.size());
  to_device(d_cm, cm.data(), cm.size());
  to_device(d_cs, cs.data(), cs.size());
  int ncl = 0;
  check(rtr_gc_group(ctx, d_mk, d_sk, d_cm, d_cs, d_cd, C, 0.01f, 5, kMaxClusters, kMaxMembers, d_mem, d_sizes, d_poses,
                     &ncl, nullptr),
        "rtr_gc_group");
  if (ncl <= 0 || ns == 0 || nm == 0) return best;
  to_device(d_s, reinterpret_cast<const float*>(cloud->points.data()), 4 * (size_t)ns);
  to_device(d_m, reinterpret_cast<const float*>(mcloud->points.data()), 4 * (size_t)nm);
  // first scores of every group's pose, on the device
  check(rtr_pose_inliers(ctx, d_m, nm, d_s, ns, d_poses, ncl, 2.f * inlier_r, d_cnt, nullptr), "rtr_pose_inliers");
  std::vector<int32_t> first((size_t)ncl);
  to_host(first.data(), d_cnt, first.size());
  std::vector<double> poses((size_t)ncl * 16);
  to_host(poses.data(), d_poses, poses.size());
  std::vector<int> order((size_t)ncl);
  for (int c = 0; c < ncl; ++c) order[(size_t)c] = c;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return first[(size_t)x] > first[(size_t)y]; });
  const int top = ncl < kTop ? ncl : kTop;
  std::vector<double> init((size_t)top * 16);
  for (int k = 0; k < top; ++k) std::memcpy(&init[(size_t)k * 16], &poses[(size_t)order[(size_t)k] * 16], 16 * sizeof(double));
  to_device(d_init, init.data(), init.size());
  // the top candidates refined together
  rtr_icp_params ip;
  rtr_icp_default_params(&ip);
  ip.max_iterations = 30;
  ip.max_corr_dist = 0.02f;
  ip.cell_size = 0.03f;
  check(rtr_icp_multi(ctx, d_m, nm, d_s, ns, &ip, d_init, top, d_res, nullptr), "rtr_icp_multi");
  std::vector<rtr_icp_result> res((size_t)top);
  to_host(res.data(), d_res, res.size());
  std::vector<double> refined((size_t)top * 16);
  for (int k = 0; k < top; ++k) std::memcpy(&refined[(size_t)k * 16], res[(size_t)k].pose, 16 * sizeof(double));
  to_device(d_init, refined.data(), refined.size());
  check(rtr_pose_inliers(ctx, d_m, nm, d_s, ns, d_init, top, inlier_r, d_cnt, nullptr), "rtr_pose_inliers");
  std::vector<int32_t> fin((size_t)top);
  to_host(fin.data(), d_cnt, fin.size());
  int w = 0;
  for (int k = 1; k < top; ++k)
    if (fin[(size_t)k] > fin[(size_t)w]) w = k;
  // model -> scene (R, t) inverted: scene -> model (R^T, -R^T t)
  const double* T = &refined[(size_t)w * 16];
  for (int r = 0; r < 3; ++r) {
    double t = 0.0;
    for (int c = 0; c < 3; ++c) {
      best(r, c) = (float)T[c * 4 + r];
      t -= T[c * 4 + r] * T[c * 4 + 3];
    }
    best(r, 3) = (float)t;
  }
  return best;
}

// function.h:111-148 without the viewer and the PCD files: ICP of mcloud
// (source) onto cloud (target) with PCL's default settings, the final
// transform printed as the reference does, and returned.  SpointCloud and
// mPointCloud are kept for the signature.
inline Eigen::Matrix4f keyPointICP_pose(Cloud::Ptr SpointCloud, Cloud::Ptr mPointCloud, Cloud::Ptr cloud, Cloud::Ptr mcloud,
                                        const Eigen::Matrix4f* init = nullptr, int max_iterations = -1,
                                        float max_corr_dist = -1.f) {
  (void)SpointCloud;
  (void)mPointCloud;
  rtr_context* ctx = thread_context();
  rtr_icp_params p;
  rtr_icp_default_params(&p);
  if (max_iterations > 0) p.max_iterations = max_iterations;
  if (max_corr_dist > 0.f) p.max_corr_dist = max_corr_dist;
  double T0[16];
  if (init)
    for (int i = 0; i < 16; ++i) T0[i] = (*init)(i / 4, i % 4);
  rtr_icp_result r;
  check(rtr_icp_host(ctx, reinterpret_cast<const float*>(mcloud->points.data()), (int)mcloud->size(),
                     reinterpret_cast<const float*>(cloud->points.data()), (int)cloud->size(), &p, init ? T0 : nullptr,
                     &r),
        "rtr_icp_host");
  Eigen::Matrix4f T;
  for (int i = 0; i < 16; ++i) T(i / 4, i % 4) = (float)r.pose[i];
  return T;
}

inline void keyPointICP(Cloud::Ptr SpointCloud, Cloud::Ptr mPointCloud, Cloud::Ptr cloud, Cloud::Ptr mcloud) {
  const Eigen::Matrix4f T = keyPointICP_pose(SpointCloud, mPointCloud, cloud, mcloud);
  std::cout << T << std::endl;
}

}  // namespace rtr_robot

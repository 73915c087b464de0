// synth.cpp — seeded synthetic point clouds (host only).
//
// Stand-ins for the reference's PCD inputs (RealTimeRobot.cpp:34-35): box
// assemblies sampled area-uniformly (chair, desk, sofa), rigid transforms with
// Gaussian noise and cropping, and a ray-cast room scene seen from one camera.
// Only integer SplitMix64 and double arithmetic are used, so a seed gives the
// same cloud on every machine up to libm's last-bit behaviour.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/rtr.h"

namespace {

struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed ^ 0x243F6A8885A308D3ull) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
  double gauss() {
    double u1 = 1.0 - uniform();  // (0,1]
    double u2 = uniform();
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
  }
};

struct Box {  // axis-aligned in the object frame
  double c[3], h[3];
};

void shape_boxes(int shape, std::vector<Box>& out) {
  out.clear();
  if (shape == 0) {  // chair: seat 0.45x0.45x0.03 on 0.45 legs, backrest at +y
    const double L = 0.225 - 0.015;
    for (int sx = -1; sx <= 1; sx += 2)
      for (int sy = -1; sy <= 1; sy += 2) out.push_back({{sx * L, sy * L, 0.225}, {0.015, 0.015, 0.225}});
    out.push_back({{0, 0, 0.465}, {0.225, 0.225, 0.015}});
    out.push_back({{0, 0.225 - 0.015, 0.705}, {0.225, 0.015, 0.225}});
  } else if (shape == 1) {  // desk: top 1.2x0.6x0.03 at 0.72..0.75 on 0.05x0.05 legs
    for (int sx = -1; sx <= 1; sx += 2)
      for (int sy = -1; sy <= 1; sy += 2)
        out.push_back({{sx * (0.6 - 0.025), sy * (0.3 - 0.025), 0.36}, {0.025, 0.025, 0.36}});
    out.push_back({{0, 0, 0.735}, {0.6, 0.3, 0.015}});
  } else {  // sofa 2.0 x 0.9 x 0.8: base, backrest, two armrests
    out.push_back({{0, 0, 0.2}, {1.0, 0.45, 0.2}});
    out.push_back({{0, 0.45 - 0.1, 0.6}, {1.0, 0.1, 0.2}});
    for (int sx = -1; sx <= 1; sx += 2) out.push_back({{sx * 0.9, -0.1, 0.5}, {0.1, 0.35, 0.1}});
  }
}

double shape_radius(int shape) { return shape == 0 ? 0.33 : (shape == 1 ? 0.68 : 1.10); }

// Area-uniform point on the faces of the boxes.
void sample_boxes(const std::vector<Box>& boxes, Rng& r, int n, float* out) {
  std::vector<double> cum;
  std::vector<int> fb, fa;  // face -> box, face -> normal axis*2+side
  double tot = 0;
  for (size_t b = 0; b < boxes.size(); ++b)
    for (int a = 0; a < 3; ++a) {
      const int u = (a + 1) % 3, v = (a + 2) % 3;
      const double area = 4.0 * boxes[b].h[u] * boxes[b].h[v];
      for (int side = 0; side < 2; ++side) {
        tot += area;
        cum.push_back(tot);
        fb.push_back((int)b);
        fa.push_back(a * 2 + side);
      }
    }
  for (int i = 0; i < n; ++i) {
    const double x = r.uniform() * tot;
    size_t f = std::upper_bound(cum.begin(), cum.end(), x) - cum.begin();
    if (f >= cum.size()) f = cum.size() - 1;
    const Box& B = boxes[fb[f]];
    const int a = fa[f] / 2, side = fa[f] % 2;
    const int u = (a + 1) % 3, v = (a + 2) % 3;
    double p[3];
    p[a] = B.c[a] + (side ? B.h[a] : -B.h[a]);
    p[u] = B.c[u] + (2.0 * r.uniform() - 1.0) * B.h[u];
    p[v] = B.c[v] + (2.0 * r.uniform() - 1.0) * B.h[v];
    out[4 * i + 0] = (float)p[0];
    out[4 * i + 1] = (float)p[1];
    out[4 * i + 2] = (float)p[2];
    out[4 * i + 3] = 0.f;
  }
}

void rot_axis_angle(const double ax[3], double ang, double R[9]) {
  const double c = cos(ang), s = sin(ang), C = 1 - c;
  const double x = ax[0], y = ax[1], z = ax[2];
  R[0] = c + x * x * C;     R[1] = x * y * C - z * s; R[2] = x * z * C + y * s;
  R[3] = y * x * C + z * s; R[4] = c + y * y * C;     R[5] = y * z * C - x * s;
  R[6] = z * x * C - y * s; R[7] = z * y * C + x * s; R[8] = c + z * z * C;
}

// Slab test of a ray (object frame) against a box; returns the entry t or -1.
double ray_box(const double o[3], const double d[3], const Box& b) {
  double t0 = -1e300, t1 = 1e300;
  for (int a = 0; a < 3; ++a) {
    const double lo = b.c[a] - b.h[a], hi = b.c[a] + b.h[a];
    if (fabs(d[a]) < 1e-15) {
      if (o[a] < lo || o[a] > hi) return -1;
      continue;
    }
    double ta = (lo - o[a]) / d[a], tb = (hi - o[a]) / d[a];
    if (ta > tb) std::swap(ta, tb);
    t0 = std::max(t0, ta);
    t1 = std::min(t1, tb);
    if (t0 > t1) return -1;
  }
  if (t1 < 1e-9) return -1;
  return t0 > 1e-9 ? t0 : -1;  // origin inside a box: no visible surface
}

struct Inst { int shape; double yaw, x, y; };

// Furniture of a room: largest first, non-overlapping bounding circles.
void place_furniture(const rtr_room_params* P, Rng& r, std::vector<Inst>& inst) {
  std::vector<int> order;
  for (int i = 0; i < P->n_sofas; ++i) order.push_back(2);
  for (int i = 0; i < P->n_desks; ++i) order.push_back(1);
  for (int i = 0; i < P->n_chairs; ++i) order.push_back(0);
  for (int sh : order) {
    const double rad = shape_radius(sh);
    for (int tries = 0; tries < 2000; ++tries) {
      const double x = -1.9 + rad * 0.5 + r.uniform() * (3.8 - rad);
      const double y = -0.6 + r.uniform() * (2.6 - rad * 0.5);
      const double yaw = 6.283185307179586 * r.uniform();
      bool ok = x - rad > -2.45 && y + rad < 2.45;
      for (const Inst& o : inst) {
        const double dx = x - o.x, dy = y - o.y;
        if (sqrt(dx * dx + dy * dy) < rad + shape_radius(o.shape) + 0.05) ok = false;
      }
      if (ok) {
        inst.push_back({sh, yaw, x, y});
        break;
      }
    }
  }
}

}  // namespace

extern "C" {

rtr_status rtr_synth_room_boxes(const rtr_room_params* P, uint64_t seed, float* h_boxes, int max_boxes,
                                int* h_n_boxes, int* h_inst_shape, double* h_inst_pose16, int max_instances,
                                int* h_n_instances) {
  if (!P || !h_boxes || !h_n_boxes) return RTR_ERR_INVALID_ARG;
  Rng r(seed);
  std::vector<Inst> inst;
  place_furniture(P, r, inst);
  int nb = 0;
  for (size_t i = 0; i < inst.size(); ++i) {
    std::vector<Box> boxes;
    shape_boxes(inst[i].shape, boxes);
    for (const Box& B : boxes) {
      if (nb >= max_boxes) return RTR_ERR_CAPACITY;
      float* o = h_boxes + 12 * nb;
      o[0] = (float)cos(inst[i].yaw);
      o[1] = (float)sin(inst[i].yaw);
      o[2] = (float)inst[i].x;
      o[3] = (float)inst[i].y;
      for (int k = 0; k < 3; ++k) {
        o[4 + k] = (float)(B.c[k] - B.h[k]);
        o[7 + k] = (float)(B.c[k] + B.h[k]);
      }
      o[10] = (float)inst[i].shape;
      o[11] = (float)i;
      ++nb;
    }
    if ((int)i < max_instances) {
      if (h_inst_shape) h_inst_shape[i] = inst[i].shape;
      if (h_inst_pose16) {
        const double c = cos(inst[i].yaw), sn = sin(inst[i].yaw);
        const double M[16] = {c, -sn, 0, inst[i].x, sn, c, 0, inst[i].y, 0, 0, 1, 0, 0, 0, 0, 1};
        memcpy(h_inst_pose16 + 16 * i, M, sizeof(M));
      }
    }
  }
  *h_n_boxes = nb;
  if (h_n_instances) *h_n_instances = (int)inst.size();
  return RTR_OK;
}

void rtr_synth_trajectory(uint64_t seed, int n_frames, double fps, double* h_poses16) {
  Rng r(seed);
  const double ph1 = 6.283185307179586 * r.uniform(), ph2 = 6.283185307179586 * r.uniform();
  const double A = 1.2, w1 = 0.5 / A;                          // x sweep, peak speed 0.5 m/s
  const double Ay = 0.349065850398866, w2 = 0.872664625997165;  // yaw +-20 deg, peak rate 17.5 deg/s
  const double pitch = -0.436332312998582;                      // 25 deg down
  for (int f = 0; f < n_frames; ++f) {
    const double t = f / fps;
    const double C[3] = {A * sin(w1 * t + ph1), -2.3 + 0.15 * sin(0.3 * t + ph2), 1.5};
    const double yaw = Ay * sin(w2 * t + ph2);
    const double fw[3] = {sin(yaw) * cos(pitch), cos(yaw) * cos(pitch), sin(pitch)};
    double rt[3] = {fw[1], -fw[0], 0.0};  // fw x (0,0,1)
    const double rn = sqrt(rt[0] * rt[0] + rt[1] * rt[1]);
    rt[0] /= rn;
    rt[1] /= rn;
    const double dn[3] = {fw[1] * rt[2] - fw[2] * rt[1], fw[2] * rt[0] - fw[0] * rt[2], fw[0] * rt[1] - fw[1] * rt[0]};
    double* T = h_poses16 + 16 * f;  // camera (x right, y down, z forward) -> world
    for (int k = 0; k < 3; ++k) {
      T[4 * k + 0] = rt[k];
      T[4 * k + 1] = dn[k];
      T[4 * k + 2] = fw[k];
      T[4 * k + 3] = C[k];
    }
    T[12] = T[13] = T[14] = 0.0;
    T[15] = 1.0;
  }
}

rtr_status rtr_synth_shape(int shape, uint64_t seed, int n, float* h_out_xyz4) {
  if (shape < 0 || shape > 2 || n < 0 || (n > 0 && !h_out_xyz4)) return RTR_ERR_INVALID_ARG;
  std::vector<Box> boxes;
  shape_boxes(shape, boxes);
  Rng r(seed);
  sample_boxes(boxes, r, n, h_out_xyz4);
  return RTR_OK;
}

void rtr_synth_rigid(uint64_t seed, double max_angle_deg, double max_t, double* T) {
  Rng r(seed ^ 0x5151A5A5ull);
  const double z = 2.0 * r.uniform() - 1.0, phi = 6.283185307179586 * r.uniform();
  const double s = sqrt(std::max(0.0, 1.0 - z * z));
  const double ax[3] = {s * cos(phi), s * sin(phi), z};
  const double ang = r.uniform() * max_angle_deg * 3.141592653589793 / 180.0;
  double R[9];
  rot_axis_angle(ax, ang, R);
  for (int i = 0; i < 3; ++i) {
    for (int j = 0; j < 3; ++j) T[i * 4 + j] = R[i * 3 + j];
    T[i * 4 + 3] = (2.0 * r.uniform() - 1.0) * max_t;
  }
  T[12] = T[13] = T[14] = 0.0;
  T[15] = 1.0;
}

void rtr_synth_transform_noise(const float* in, int n, const double* T, double sigma, uint64_t seed,
                               float* out) {
  Rng r(seed ^ 0xC0FFEEull);
  for (int i = 0; i < n; ++i) {
    const double x = in[4 * i], y = in[4 * i + 1], z = in[4 * i + 2];
    double q[3];
    for (int a = 0; a < 3; ++a) q[a] = T[a * 4] * x + T[a * 4 + 1] * y + T[a * 4 + 2] * z + T[a * 4 + 3];
    for (int a = 0; a < 3; ++a) {
      const double nz = sigma > 0 ? sigma * r.gauss() : 0.0;
      out[4 * i + a] = (float)(q[a] + nz);
    }
    out[4 * i + 3] = 0.f;
  }
}

int rtr_synth_crop(const float* in, int n, double max_frac, uint64_t seed, float* out) {
  Rng r(seed ^ 0xC409ull);
  const double frac = r.uniform() * max_frac;
  const double z = 2.0 * r.uniform() - 1.0, phi = 6.283185307179586 * r.uniform();
  const double s = sqrt(std::max(0.0, 1.0 - z * z));
  const double u[3] = {s * cos(phi), s * sin(phi), z};
  std::vector<std::pair<double, int>> proj((size_t)n);
  for (int i = 0; i < n; ++i) proj[i] = {u[0] * in[4 * i] + u[1] * in[4 * i + 1] + u[2] * in[4 * i + 2], i};
  std::sort(proj.begin(), proj.end());
  const int keep = n - (int)floor(frac * n);
  std::vector<char> keepm((size_t)n, 0);
  for (int i = 0; i < keep; ++i) keepm[proj[i].second] = 1;
  int m = 0;
  for (int i = 0; i < n; ++i)
    if (keepm[i]) {
      memmove(out + 4 * m, in + 4 * i, 16);
      ++m;
    }
  return m;
}

void rtr_room_default_params(rtr_room_params* p) {
  p->n_points = 300000;
  p->n_chairs = 3;
  p->n_desks = 1;
  p->n_sofas = 0;
  p->sigma = 0.003;
  p->cam[0] = 0.0; p->cam[1] = -2.5; p->cam[2] = 1.5;
  p->look_at[0] = 0.0; p->look_at[1] = 0.8; p->look_at[2] = 0.3;
  p->width = 640;
  p->height = 480;
  p->fx = p->fy = 400.0;
  p->cx = 319.5;
  p->cy = 239.5;
}

rtr_status rtr_synth_room(const rtr_room_params* P, uint64_t seed, float* out, int max_instances,
                          int* inst_shape, double* inst_pose, int* n_instances) {
  if (!P || !out || P->n_points < 0) return RTR_ERR_INVALID_ARG;
  Rng r(seed);
  std::vector<Inst> inst;
  place_furniture(P, r, inst);
  std::vector<std::vector<Box>> boxes(inst.size());
  for (size_t i = 0; i < inst.size(); ++i) shape_boxes(inst[i].shape, boxes[i]);
  if (n_instances) *n_instances = (int)inst.size();
  for (size_t i = 0; i < inst.size() && (int)i < max_instances; ++i) {
    if (inst_shape) inst_shape[i] = inst[i].shape;
    if (inst_pose) {
      const double c = cos(inst[i].yaw), s = sin(inst[i].yaw);
      double* T = inst_pose + 16 * i;
      const double M[16] = {c, -s, 0, inst[i].x, s, c, 0, inst[i].y, 0, 0, 1, 0, 0, 0, 0, 1};
      memcpy(T, M, sizeof(M));
    }
  }
  // camera frame
  double f[3] = {P->look_at[0] - P->cam[0], P->look_at[1] - P->cam[1], P->look_at[2] - P->cam[2]};
  double fn = sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
  for (double& v : f) v /= fn;
  double rt[3] = {f[1] * 1.0 - f[2] * 0.0, f[2] * 0.0 - f[0] * 1.0, 0.0};  // f x (0,0,1)
  double rn = sqrt(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2]);
  for (double& v : rt) v /= rn;
  const double dn[3] = {f[1] * rt[2] - f[2] * rt[1], f[2] * rt[0] - f[0] * rt[2], f[0] * rt[1] - f[1] * rt[0]};
  const double* C = P->cam;
  int m = 0;
  long long guard = 0;
  while (m < P->n_points && guard < 50LL * (P->n_points + 1)) {
    ++guard;
    const double u = r.uniform() * P->width, v = r.uniform() * P->height;
    const double a = (u - P->cx) / P->fx, b = (v - P->cy) / P->fy;
    double d[3];
    for (int k = 0; k < 3; ++k) d[k] = f[k] + a * rt[k] + b * dn[k];
    const double dl = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    for (double& w : d) w /= dl;
    double tbest = 1e300;
    // floor z = 0
    if (d[2] < -1e-12) {
      const double t = -C[2] / d[2];
      const double x = C[0] + t * d[0], y = C[1] + t * d[1];
      if (fabs(x) <= 2.5 && fabs(y) <= 2.5 && t < tbest) tbest = t;
    }
    // back wall y = 2.5
    if (d[1] > 1e-12) {
      const double t = (2.5 - C[1]) / d[1];
      const double x = C[0] + t * d[0], z = C[2] + t * d[2];
      if (fabs(x) <= 2.5 && z >= 0 && z <= 3.0 && t < tbest) tbest = t;
    }
    // left wall x = -2.5
    if (d[0] < -1e-12) {
      const double t = (-2.5 - C[0]) / d[0];
      const double y = C[1] + t * d[1], z = C[2] + t * d[2];
      if (fabs(y) <= 2.5 && z >= 0 && z <= 3.0 && t < tbest) tbest = t;
    }
    for (size_t i = 0; i < inst.size(); ++i) {
      const double c = cos(inst[i].yaw), s = sin(inst[i].yaw);
      const double ow[3] = {C[0] - inst[i].x, C[1] - inst[i].y, C[2]};
      const double o[3] = {c * ow[0] + s * ow[1], -s * ow[0] + c * ow[1], ow[2]};
      const double dd[3] = {c * d[0] + s * d[1], -s * d[0] + c * d[1], d[2]};
      for (const Box& B : boxes[i]) {
        const double t = ray_box(o, dd, B);
        if (t > 0 && t < tbest) tbest = t;
      }
    }
    if (tbest >= 1e299) continue;
    for (int k = 0; k < 3; ++k) out[4 * m + k] = (float)(C[k] + tbest * d[k] + P->sigma * r.gauss());
    out[4 * m + 3] = 0.f;
    ++m;
  }
  if (m < P->n_points) return RTR_ERR_INVALID_ARG;
  return RTR_OK;
}

}  // extern "C"

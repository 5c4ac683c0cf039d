// sgba_synth.cpp -- seeded synthetic bundle-adjustment scenes (host only).
//
// Plays the role of the reference's example-problem generators
// (crates/sophus_opt/src/example_problems/ba_problem.rs:154-346): ground-truth
// cameras and points, noisy pixel observations, perturbed initial values.
// Geometry follows the benchmark configurations: a circle of cameras around a
// cube, a Fibonacci sphere of cameras with random track subsets, and a long
// outward-facing loop whose points are seen by runs of consecutive cameras.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/sgba_synth.h"

namespace {

// SplitMix64 (Steele, Lea, Flood 2014) -- one independent stream per purpose.
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed, uint64_t stream) : s(seed ^ (0xD1B54A32D192ED03ull * (stream + 1))) {
    next(); next();
  }
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }  // [0,1)
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  int uniform_int(int lo, int hi) {  // inclusive
    uint64_t span = static_cast<uint64_t>(hi - lo + 1);
    return lo + static_cast<int>(next() % span);
  }
  // Box-Muller (cosine branch)
  double normal(double sigma) {
    double u1 = 1.0 - uniform();  // (0,1]
    double u2 = uniform();
    return sigma * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
  }
};

struct Pose {  // world_from_camera
  double q[4];  // w x y z
  double t[3];
};

void quat_from_matrix(const double* m, double* q) {  // row-major rotation
  double tr = m[0] + m[4] + m[8];
  double w, x, y, z;
  if (tr > 0.0) {
    double s = std::sqrt(tr + 1.0) * 2.0;
    w = 0.25 * s; x = (m[7] - m[5]) / s; y = (m[2] - m[6]) / s; z = (m[3] - m[1]) / s;
  } else if (m[0] > m[4] && m[0] > m[8]) {
    double s = std::sqrt(1.0 + m[0] - m[4] - m[8]) * 2.0;
    w = (m[7] - m[5]) / s; x = 0.25 * s; y = (m[1] + m[3]) / s; z = (m[2] + m[6]) / s;
  } else if (m[4] > m[8]) {
    double s = std::sqrt(1.0 + m[4] - m[0] - m[8]) * 2.0;
    w = (m[2] - m[6]) / s; x = (m[1] + m[3]) / s; y = 0.25 * s; z = (m[5] + m[7]) / s;
  } else {
    double s = std::sqrt(1.0 + m[8] - m[0] - m[4]) * 2.0;
    w = (m[3] - m[1]) / s; x = (m[2] + m[6]) / s; y = (m[5] + m[7]) / s; z = 0.25 * s;
  }
  double n = std::sqrt(w * w + x * x + y * y + z * z);
  if (w < 0.0) n = -n;
  q[0] = w / n; q[1] = x / n; q[2] = y / n; q[3] = z / n;
}

void rot_from_quat(const double* q, double* m) {
  double w = q[0], x = q[1], y = q[2], z = q[3];
  m[0] = 1 - 2 * (y * y + z * z); m[1] = 2 * (x * y - w * z); m[2] = 2 * (x * z + w * y);
  m[3] = 2 * (x * y + w * z); m[4] = 1 - 2 * (x * x + z * z); m[5] = 2 * (y * z - w * x);
  m[6] = 2 * (x * z - w * y); m[7] = 2 * (y * z + w * x); m[8] = 1 - 2 * (x * x + y * y);
}

void normalize3(double* v) {
  double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  v[0] /= n; v[1] /= n; v[2] /= n;
}
void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// Camera at `c` with optical axis `f` (z forward, x right, y down; world z up).
Pose camera_along(const double* c, const double* fwd) {
  double f[3] = {fwd[0], fwd[1], fwd[2]};
  normalize3(f);
  double up[3] = {0.0, 0.0, 1.0};
  double r[3];
  cross3(f, up, r);
  if (std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) < 1e-6) {
    double up2[3] = {0.0, 1.0, 0.0};
    cross3(f, up2, r);
  }
  normalize3(r);
  double d[3];
  cross3(f, r, d);
  double m[9] = {r[0], d[0], f[0], r[1], d[1], f[1], r[2], d[2], f[2]};
  Pose p;
  quat_from_matrix(m, p.q);
  p.t[0] = c[0]; p.t[1] = c[1]; p.t[2] = c[2];
  return p;
}

Pose look_at(const double* c, const double* target) {
  double f[3] = {target[0] - c[0], target[1] - c[1], target[2] - c[2]};
  return camera_along(c, f);
}

constexpr double kFx = 500.0, kFy = 500.0, kCx = 320.0, kCy = 240.0;
constexpr double kW = 640.0, kH = 480.0;

// Project world point through camera; true if depth > 0.1 and inside the image.
bool project(const Pose& p, const double* x, double* uv) {
  double r[9];
  rot_from_quat(p.q, r);
  double d[3] = {x[0] - p.t[0], x[1] - p.t[1], x[2] - p.t[2]};
  double xc[3];
  for (int i = 0; i < 3; ++i) xc[i] = r[0 * 3 + i] * d[0] + r[1 * 3 + i] * d[1] + r[2 * 3 + i] * d[2];
  if (!(xc[2] > 0.1)) return false;
  uv[0] = kFx * xc[0] / xc[2] + kCx;
  uv[1] = kFy * xc[1] / xc[2] + kCy;
  return uv[0] >= 0.0 && uv[0] < kW && uv[1] >= 0.0 && uv[1] < kH;
}

// Left perturbation exp([w; v]) * T (first-order-exact SE(3) exponential).
Pose perturb(const Pose& p, Rng& rng, double sig_rot, double sig_trans) {
  double w[3] = {rng.normal(sig_rot), rng.normal(sig_rot), rng.normal(sig_rot)};
  double v[3] = {rng.normal(sig_trans), rng.normal(sig_trans), rng.normal(sig_trans)};
  double th = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  double dq[4];
  if (th < 1e-12) {
    dq[0] = 1.0; dq[1] = 0.5 * w[0]; dq[2] = 0.5 * w[1]; dq[3] = 0.5 * w[2];
  } else {
    double s = std::sin(0.5 * th) / th;
    dq[0] = std::cos(0.5 * th); dq[1] = s * w[0]; dq[2] = s * w[1]; dq[3] = s * w[2];
  }
  // V(w) * v
  double tv[3];
  {
    double h[9] = {0, -w[2], w[1], w[2], 0, -w[0], -w[1], w[0], 0};
    double h2[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        h2[i * 3 + j] = h[i * 3 + 0] * h[0 * 3 + j] + h[i * 3 + 1] * h[1 * 3 + j] + h[i * 3 + 2] * h[2 * 3 + j];
    double a = 0.5, b = 1.0 / 6.0;
    if (th > 1e-6) { a = (1 - std::cos(th)) / (th * th); b = (th - std::sin(th)) / (th * th * th); }
    for (int i = 0; i < 3; ++i) {
      double row[3];
      for (int j = 0; j < 3; ++j) row[j] = (i == j ? 1.0 : 0.0) + a * h[i * 3 + j] + b * h2[i * 3 + j];
      tv[i] = row[0] * v[0] + row[1] * v[1] + row[2] * v[2];
    }
  }
  Pose o;
  const double* a = dq;
  const double* b = p.q;
  o.q[0] = a[0] * b[0] - (a[1] * b[1] + a[2] * b[2] + a[3] * b[3]);
  o.q[1] = b[1] * a[0] + a[1] * b[0] + (a[2] * b[3] - a[3] * b[2]);
  o.q[2] = b[2] * a[0] + a[2] * b[0] + (a[3] * b[1] - a[1] * b[3]);
  o.q[3] = b[3] * a[0] + a[3] * b[0] + (a[1] * b[2] - a[2] * b[1]);
  double n = std::sqrt(o.q[0] * o.q[0] + o.q[1] * o.q[1] + o.q[2] * o.q[2] + o.q[3] * o.q[3]);
  if (o.q[0] < 0) n = -n;
  for (int i = 0; i < 4; ++i) o.q[i] /= n;
  double r[9];
  rot_from_quat(dq, r);
  for (int i = 0; i < 3; ++i)
    o.t[i] = r[i * 3 + 0] * p.t[0] + r[i * 3 + 1] * p.t[1] + r[i * 3 + 2] * p.t[2] + tv[i];
  return o;
}

struct Scene {
  std::vector<Pose> cams;
  std::vector<double> pts;  // 3 per point
  std::vector<int32_t> ocam, opt;
  std::vector<double> ouv;
};

// Cameras on a circle of radius r at height h looking at the origin; points
// uniform in [-e, e]^3; every camera that sees a point observes it.
void circle_scene(Scene* s, int n_cam, int n_pt, double radius, double height, double extent,
                  Rng& geo, Rng& noise) {
  for (int j = 0; j < n_cam; ++j) {
    double a = 6.283185307179586 * j / n_cam;
    double c[3] = {radius * std::cos(a), radius * std::sin(a), height};
    double o[3] = {0, 0, 0};
    s->cams.push_back(look_at(c, o));
  }
  for (int i = 0; i < n_pt; ++i) {
    for (;;) {
      double x[3] = {geo.uniform(-extent, extent), geo.uniform(-extent, extent), geo.uniform(-extent, extent)};
      std::vector<std::pair<int, std::pair<double, double>>> seen;
      for (int j = 0; j < n_cam; ++j) {
        double uv[2];
        if (project(s->cams[j], x, uv)) seen.push_back({j, {uv[0], uv[1]}});
      }
      if (seen.size() < 2) continue;  // a point needs two views to be constrained
      for (auto& e : seen) {
        s->ocam.push_back(e.first);
        s->opt.push_back(static_cast<int32_t>(s->pts.size() / 3));
        s->ouv.push_back(e.second.first + noise.normal(0.5));
        s->ouv.push_back(e.second.second + noise.normal(0.5));
      }
      s->pts.insert(s->pts.end(), x, x + 3);
      break;
    }
  }
}

// Fibonacci sphere of cameras (radius r) looking at the origin; points uniform
// in [-e, e]^3, each observed by k ~ U{kmin..kmax} of the cameras that see it.
void sphere_scene(Scene* s, int n_cam, int n_pt, double radius, double extent, int kmin, int kmax,
                  Rng& geo, Rng& pick, Rng& noise) {
  const double golden = 3.141592653589793 * (3.0 - std::sqrt(5.0));
  for (int j = 0; j < n_cam; ++j) {
    double z = 1.0 - 2.0 * (j + 0.5) / n_cam;
    double rr = std::sqrt(std::max(0.0, 1.0 - z * z));
    double phi = golden * j;
    double c[3] = {radius * rr * std::cos(phi), radius * rr * std::sin(phi), radius * z};
    double o[3] = {0, 0, 0};
    s->cams.push_back(look_at(c, o));
  }
  std::vector<int> vis;
  std::vector<double> vuv;
  for (int i = 0; i < n_pt; ++i) {
    for (;;) {
      double x[3] = {geo.uniform(-extent, extent), geo.uniform(-extent, extent), geo.uniform(-extent, extent)};
      vis.clear(); vuv.clear();
      for (int j = 0; j < n_cam; ++j) {
        double uv[2];
        if (project(s->cams[j], x, uv)) { vis.push_back(j); vuv.push_back(uv[0]); vuv.push_back(uv[1]); }
      }
      if (vis.size() < 2) continue;
      int k = std::min<int>(pick.uniform_int(kmin, kmax), static_cast<int>(vis.size()));
      std::vector<int> idx(vis.size());
      for (size_t t = 0; t < idx.size(); ++t) idx[t] = static_cast<int>(t);
      for (int t = 0; t < k; ++t) {  // partial Fisher-Yates
        int u = t + static_cast<int>(pick.next() % static_cast<uint64_t>(idx.size() - t));
        std::swap(idx[t], idx[u]);
      }
      std::sort(idx.begin(), idx.begin() + k);
      int pid = static_cast<int>(s->pts.size() / 3);
      for (int t = 0; t < k; ++t) {
        s->ocam.push_back(vis[idx[t]]);
        s->opt.push_back(pid);
        s->ouv.push_back(vuv[2 * idx[t]] + noise.normal(0.5));
        s->ouv.push_back(vuv[2 * idx[t] + 1] + noise.normal(0.5));
      }
      s->pts.insert(s->pts.end(), x, x + 3);
      break;
    }
  }
}

// Outward-facing loop of cameras (radius r, radial jitter); points on a
// cylinder wall (radius rc, height in [-h, h]) seen by a run of consecutive
// cameras whose length is geometric(p) clipped to [lmin, lmax].
void loop_scene(Scene* s, int n_cam, int n_pt, double radius, double jitter, double rc, double h,
                double p, int lmin, int lmax, Rng& geo, Rng& pick, Rng& noise) {
  for (int j = 0; j < n_cam; ++j) {
    double a = 6.283185307179586 * j / n_cam;
    double rad = radius + geo.normal(jitter);
    double c[3] = {rad * std::cos(a), rad * std::sin(a), 0.0};
    double f[3] = {std::cos(a), std::sin(a), 0.0};
    s->cams.push_back(camera_along(c, f));
  }
  const double step = 6.283185307179586 / n_cam;
  for (int i = 0; i < n_pt; ++i) {
    for (;;) {
      int start = pick.uniform_int(0, n_cam - 1);
      // geometric number of trials to first success, clipped
      int len = 1;
      while (pick.uniform() >= p && len < 10000) ++len;
      len = std::max(lmin, std::min(lmax, len));
      double mid = (start + 0.5 * (len - 1)) * step;
      double ang = mid + geo.uniform(-0.5, 0.5) * step;
      double x[3] = {rc * std::cos(ang), rc * std::sin(ang), geo.uniform(-h, h)};
      int pid = static_cast<int>(s->pts.size() / 3);
      size_t before = s->ocam.size();
      for (int t = 0; t < len; ++t) {
        int j = (start + t) % n_cam;
        double uv[2];
        if (!project(s->cams[j], x, uv)) continue;
        s->ocam.push_back(j);
        s->opt.push_back(pid);
        s->ouv.push_back(uv[0] + noise.normal(0.5));
        s->ouv.push_back(uv[1] + noise.normal(0.5));
      }
      if (s->ocam.size() - before < 2) {  // need two views; redraw the point
        s->ocam.resize(before); s->opt.resize(before); s->ouv.resize(2 * before);
        continue;
      }
      s->pts.insert(s->pts.end(), x, x + 3);
      break;
    }
  }
}

template <class T>
T* dup(const std::vector<T>& v) {
  T* p = static_cast<T*>(std::malloc(sizeof(T) * std::max<size_t>(v.size(), 1)));
  if (p && !v.empty()) std::memcpy(p, v.data(), sizeof(T) * v.size());
  return p;
}

}  // namespace

extern "C" int sgba_synth_generate(int32_t kind, int32_t n_cam, int32_t n_pt, uint64_t seed,
                                   sgba_synth_problem** out) {
  if (!out) return -1;
  *out = nullptr;
  Rng geo(seed, 0), pick(seed, 1), noise(seed, 2), pert(seed, 3), sizes(seed, 4);
  Scene s;
  int iters = 10;
  switch (kind) {
    case SGBA_SYNTH_CIRCLE:
      if (n_cam <= 0) n_cam = 10;
      if (n_pt <= 0) n_pt = 500;
      circle_scene(&s, n_cam, n_pt, 4.0, 0.5, 1.0, geo, noise);
      iters = 10;
      break;
    case SGBA_SYNTH_SPHERE:
      if (n_cam <= 0) n_cam = 100;
      if (n_pt <= 0) n_pt = 20000;
      sphere_scene(&s, n_cam, n_pt, 6.0, 2.0, 10, 40, geo, pick, noise);
      iters = 20;
      break;
    case SGBA_SYNTH_LOOP:
      if (n_cam <= 0) n_cam = 1500;
      if (n_pt <= 0) n_pt = 300000;
      loop_scene(&s, n_cam, n_pt, 50.0, 0.2, 60.0, 5.0, 0.12, 3, 25, geo, pick, noise);
      iters = 15;
      break;
    case SGBA_SYNTH_WINDOW:
      if (n_cam <= 0) n_cam = sizes.uniform_int(5, 40);
      if (n_pt <= 0) n_pt = sizes.uniform_int(200, 4000);
      circle_scene(&s, n_cam, n_pt, 4.0, 0.5, 1.0, geo, noise);
      iters = 10;
      break;
    default:
      return -2;
  }
  if (n_cam < 2 || n_pt < 1) return -3;
  sgba_synth_problem* p = static_cast<sgba_synth_problem*>(std::calloc(1, sizeof(sgba_synth_problem)));
  if (!p) return -4;
  p->n_cam = n_cam;
  p->n_pt = n_pt;
  p->n_obs = static_cast<int64_t>(s.ocam.size());
  p->intrinsics[0] = kFx; p->intrinsics[1] = kFy; p->intrinsics[2] = kCx; p->intrinsics[3] = kCy;
  p->huber_delta = 1.0;
  p->initial_lm_damping = 1e-4;
  p->num_iterations = iters;
  std::vector<double> pt(7 * n_cam), pi(7 * n_cam);
  std::vector<uint8_t> pc(n_cam, 0);
  pc[0] = 1;
  for (int j = 0; j < n_cam; ++j) {
    const Pose& t = s.cams[j];
    Pose q = (j == 0) ? t : perturb(t, pert, 0.02, 0.05);
    for (int k = 0; k < 4; ++k) { pt[7 * j + k] = t.q[k]; pi[7 * j + k] = q.q[k]; }
    for (int k = 0; k < 3; ++k) { pt[7 * j + 4 + k] = t.t[k]; pi[7 * j + 4 + k] = q.t[k]; }
  }
  std::vector<double> ptsi(s.pts.size());
  for (size_t k = 0; k < s.pts.size(); ++k) ptsi[k] = s.pts[k] + pert.normal(0.05);
  p->poses = dup(pi);
  p->poses_true = dup(pt);
  p->pose_const = dup(pc);
  p->points = dup(ptsi);
  p->points_true = dup(s.pts);
  p->obs_cam = dup(s.ocam);
  p->obs_pt = dup(s.opt);
  p->obs_uv = dup(s.ouv);
  *out = p;
  return 0;
}

extern "C" void sgba_synth_free(sgba_synth_problem* p) {
  if (!p) return;
  std::free(p->poses); std::free(p->poses_true); std::free(p->pose_const);
  std::free(p->points); std::free(p->points_true);
  std::free(p->obs_cam); std::free(p->obs_pt); std::free(p->obs_uv);
  std::free(p);
}

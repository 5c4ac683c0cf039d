// C++ tests of the sophus_opt mirror (host/sophus_opt.hpp) on the GPU backend,
// restating the reference's own tests for this path:
//   simple_cam_tests, marginalized-points variant
//     (crates/sophus_opt/src/example_problems/cam_calib.rs:244-300, 348-365)
//   ba_converges, Schur variant (crates/sophus_opt/src/example_problems/ba_problem.rs:517-547)
//   solver_validation "death tests" (crates/sophus_opt/src/example_problems/solver_validation.rs:185-365)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <string>
#include <vector>

#include "host/sophus_opt.hpp"
#include "sgba_synth.h"

using namespace sgba::opt;

static int g_fail = 0;
#define EXPECT(cond, msg)                                                   \
  do {                                                                      \
    if (!(cond)) {                                                          \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, std::string(msg).c_str()); \
      ++g_fail;                                                             \
    }                                                                       \
  } while (0)

struct Rng {  // SplitMix64
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  double uniform() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return static_cast<double>(z >> 11) * 0x1.0p-53;
  }
};

// Three cameras translated along y, 40 points at depth 10 in camera 0,
// cameras 0 and 1 fixed, camera 2 initialised at camera 1's pose.
static void simple_cam_marg_points() {
  const double fx = 600, fy = 600, cx = 320, cy = 240;
  std::vector<Isometry3F64> truth(3);
  truth[1].params[5] = 1.0;
  truth[2].params[5] = 2.0;
  Rng rng(7);
  std::vector<VecF64_3> pts;
  std::vector<PinholeCameraReprojectionCostTerm> obs;
  for (size_t i = 0; i < 40; ++i) {
    double u = rng.uniform() * 639.0, v = rng.uniform() * 479.0;
    VecF64_3 p{(u - cx) / fx * 10.0, (v - cy) / fy * 10.0, 10.0};
    pts.push_back(p);
    for (size_t c = 0; c < 3; ++c) {
      // world_from_camera is a pure translation: x_cam = p - t
      double xc = p[0] - truth[c].params[4], yc = p[1] - truth[c].params[5], zc = p[2] - truth[c].params[6];
      double nu = rng.uniform() - 0.5, nv = rng.uniform() - 0.5;
      obs.push_back({{fx * xc / zc + cx + nu, fy * yc / zc + cy + nv}, {0, c, i}});
    }
  }
  std::vector<Isometry3F64> init{truth[0], truth[1], truth[1]};
  VarFamilies vars = VarBuilder::new_()
                         .add_family("cams", VarFamily<PinholeCameraF64>::new_(
                                                 VarKind::Conditioned, {PinholeCameraF64{{fx, fy, cx, cy}, {640, 480}}}))
                         .add_family("poses", VarFamily<Isometry3F64>::new_with_const_ids(VarKind::Free, init, {0, 1}))
                         .add_family("points", VarFamily<VecF64_3>::new_(VarKind::Marginalized, pts))
                         .build();
  OptParams params;
  params.num_iterations = 25;
  params.initial_lm_damping = 1.0;
  params.parallelize = false;
  params.solver = LinearSolverEnum::SchurBlockSparseLdlt;
  auto sol = optimize_nlls(vars, {CostFn::new_boxed_robust(CostTerms::new_({"cams", "poses", "points"}, obs),
                                                           HuberKernel::new_(1.0))},
                           {}, params, 0);
  auto t = sol.variables.get_members<Isometry3F64>("poses")[2].translation();
  EXPECT(std::fabs(t[0] - 0.0) < 0.1 && std::fabs(t[1] - 2.0) < 0.1 && std::fabs(t[2] - 0.0) < 0.1,
         "camera 2 translation " + std::to_string(t[0]) + "," + std::to_string(t[1]) + "," + std::to_string(t[2]));
  std::printf("OK simple_cam_marg_points (t2 = %.4f %.4f %.4f, cost %.4f, %zu steps)\n", t[0], t[1], t[2],
              sol.final_cost, sol.steps.size());
  // covariance / precision queries by family name (OptimizationSolution::covariance_block)
  auto c22 = sol.covariance_block("poses", 2, "poses", 2);
  EXPECT(c22 && c22->rows == 6 && c22->cols == 6, "pose 2 covariance block");
  if (c22) {
    bool sym = true, pos = true;
    for (int a = 0; a < 6; ++a) {
      pos = pos && c22->values[a * 6 + a] > 0.0;
      for (int b = 0; b < 6; ++b)
        sym = sym && std::fabs(c22->values[a * 6 + b] - c22->values[b * 6 + a]) <= 1e-12 * std::fabs(c22->values[a * 6 + a]);
    }
    EXPECT(sym && pos, "pose 2 covariance is symmetric with a positive diagonal");
  }
  auto c2p = sol.covariance_block("poses", 2, "points", 0);
  EXPECT(c2p && c2p->rows == 6 && c2p->cols == 3, "pose x point covariance block");
  auto h22 = sol.precision_block("poses", 2, "poses", 2);
  EXPECT(h22 && h22->rows == 6 && h22->values[0] > 0.0, "pose 2 precision block");
  EXPECT(!sol.covariance_block("poses", 0, "poses", 2), "a constant pose has no block");
  EXPECT(!sol.covariance_block("cams", 0, "poses", 2), "the Conditioned camera family has no block");
  std::printf("OK covariance queries (var t2_x %.3e)\n", c22 ? c22->values[21] : 0.0);
}

// Circle scene; converge to the ground truth up to the scale gauge about
// the fixed camera 0.
static void ba_converges() {
  sgba_synth_problem* s = nullptr;
  if (sgba_synth_generate(SGBA_SYNTH_CIRCLE, 4, 20, 20261203, &s) != 0) {
    EXPECT(false, "synth");
    return;
  }
  std::vector<Isometry3F64> poses(s->n_cam);
  for (int j = 0; j < s->n_cam; ++j)
    for (int k = 0; k < 7; ++k) poses[j].params[k] = s->poses[7 * j + k];
  std::vector<VecF64_3> pts(s->n_pt);
  for (int i = 0; i < s->n_pt; ++i)
    for (int k = 0; k < 3; ++k) pts[i][k] = s->points[3 * i + k];
  // noise-free pixels at the ground truth plus the reference's pixel noise
  // 0.15 * U(-0.5, 0.5) (ba_problem.rs:251-253)
  std::vector<PinholeCameraReprojectionCostTerm> obs;
  Rng rng(3);
  for (int64_t o = 0; o < s->n_obs; ++o) {
    const double* T = s->poses_true + 7 * s->obs_cam[o];
    const double* p = s->points_true + 3 * s->obs_pt[o];
    const double w = T[0], x = T[1], y = T[2], z = T[3];
    const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y),
                         2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                         2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)};
    double d[3] = {p[0] - T[4], p[1] - T[5], p[2] - T[6]}, xc[3];
    for (int i = 0; i < 3; ++i) xc[i] = R[0 * 3 + i] * d[0] + R[1 * 3 + i] * d[1] + R[2 * 3 + i] * d[2];
    double u = s->intrinsics[0] * xc[0] / xc[2] + s->intrinsics[2] + 0.15 * (rng.uniform() - 0.5);
    double v = s->intrinsics[1] * xc[1] / xc[2] + s->intrinsics[3] + 0.15 * (rng.uniform() - 0.5);
    obs.push_back({{u, v}, {0, static_cast<size_t>(s->obs_cam[o]), static_cast<size_t>(s->obs_pt[o])}});
  }
  PinholeCameraF64 cam{{s->intrinsics[0], s->intrinsics[1], s->intrinsics[2], s->intrinsics[3]}, {640, 480}};
  VarFamilies vars = VarBuilder::new_()
                         .add_family("cams", VarFamily<PinholeCameraF64>::new_(VarKind::Conditioned, {cam}))
                         .add_family("poses", VarFamily<Isometry3F64>::new_with_const_ids(VarKind::Free, poses, {0}))
                         .add_family("points", VarFamily<VecF64_3>::new_(VarKind::Marginalized, pts))
                         .build();
  OptParams params;
  params.num_iterations = 30;
  params.initial_lm_damping = 1.0;
  params.solver = LinearSolverEnum::SchurBlockSparseLdlt;
  auto sol = optimize_nlls(vars, {CostFn::new_boxed_robust(CostTerms::new_({"cams", "poses", "points"}, obs),
                                                           HuberKernel::new_(1.0))},
                           {}, params, 0);
  const auto& rp = sol.variables.get_members<Isometry3F64>("poses");
  const auto& rq = sol.variables.get_members<VecF64_3>("points");
  // best scale about camera 0's center
  const double* c0 = s->poses_true + 4;
  double num = 0, den = 0;
  for (int i = 0; i < s->n_pt; ++i)
    for (int k = 0; k < 3; ++k) {
      num += (rq[i][k] - c0[k]) * (s->points_true[3 * i + k] - c0[k]);
      den += (rq[i][k] - c0[k]) * (rq[i][k] - c0[k]);
    }
  const double sc = num / den;
  double pose_se = 0, pt_se = 0;
  for (int j = 0; j < s->n_cam; ++j)
    for (int k = 0; k < 3; ++k) {
      double e = c0[k] + sc * (rp[j].params[4 + k] - c0[k]) - s->poses_true[7 * j + 4 + k];
      pose_se += e * e;
    }
  for (int i = 0; i < s->n_pt; ++i)
    for (int k = 0; k < 3; ++k) {
      double e = c0[k] + sc * (rq[i][k] - c0[k]) - s->points_true[3 * i + k];
      pt_se += e * e;
    }
  const double pose_rms = std::sqrt(pose_se / s->n_cam), pt_rms = std::sqrt(pt_se / s->n_pt);
  EXPECT(pose_rms < 0.01, "pose rms " + std::to_string(pose_rms));
  EXPECT(pt_rms < 0.1, "point rms " + std::to_string(pt_rms));
  std::printf("OK ba_converges (pose rms %.5f, point rms %.5f, scale %.6f)\n", pose_rms, pt_rms, sc);
  sgba_synth_free(s);
}

template <class E>
static bool throws(const std::function<void()>& f) {
  try {
    f();
  } catch (const E&) {
    return true;
  } catch (...) {
    return false;
  }
  return false;
}

static void solver_validation() {
  PinholeCameraF64 cam{{500, 500, 320, 240}, {640, 480}};
  std::vector<Isometry3F64> poses(2);
  poses[1].params[4] = 1.0;
  std::vector<VecF64_3> pts{{0, 0, 5}};
  std::vector<PinholeCameraReprojectionCostTerm> obs{{{320, 240}, {0, 0, 0}}, {{220, 240}, {0, 1, 0}}};
  OptParams params;
  params.solver = LinearSolverEnum::SchurBlockSparseLdlt;
  auto terms = CostTerms::new_({"cams", "poses", "points"}, obs);
  // no marginalized family -> SchurMissingFreeOrMarg
  auto v1 = VarBuilder::new_()
                .add_family("cams", VarFamily<PinholeCameraF64>::new_(VarKind::Conditioned, {cam}))
                .add_family("poses", VarFamily<Isometry3F64>::new_(VarKind::Free, poses))
                .add_family("points", VarFamily<VecF64_3>::new_(VarKind::Free, pts))
                .build();
  EXPECT(throws<SchurMissingFreeOrMarg>([&] { optimize_nlls(v1, {CostFn::new_boxed(terms)}, {}, params, 0); }),
         "missing marg");
  // two marginalized families in one cost -> SchurCostConnectsTwoMargFamilies
  auto v2 = VarBuilder::new_()
                .add_family("cams", VarFamily<PinholeCameraF64>::new_(VarKind::Free, {cam}))
                .add_family("poses", VarFamily<Isometry3F64>::new_(VarKind::Marginalized, poses))
                .add_family("points", VarFamily<VecF64_3>::new_(VarKind::Marginalized, pts))
                .build();
  EXPECT(throws<SchurCostConnectsTwoMargFamilies>(
             [&] { optimize_nlls(v2, {CostFn::new_boxed(terms)}, {}, params, 0); }),
         "two marg families");
  // non-Schur solver -> not this path
  OptParams p3;
  EXPECT(throws<NotOnGpuPath>([&] {
           auto v = VarBuilder::new_()
                        .add_family("cams", VarFamily<PinholeCameraF64>::new_(VarKind::Conditioned, {cam}))
                        .add_family("poses", VarFamily<Isometry3F64>::new_(VarKind::Free, poses))
                        .add_family("points", VarFamily<VecF64_3>::new_(VarKind::Marginalized, pts))
                        .build();
           optimize_nlls(v, {CostFn::new_boxed(terms)}, {}, p3, 0);
         }),
         "non-Schur solver");
  std::printf("OK solver_validation\n");
}

// Optimizer::step three times == optimize_nlls with three iterations.
static void stepper_matches_optimize() {
  sgba_synth_problem* s = nullptr;
  sgba_synth_generate(SGBA_SYNTH_CIRCLE, 6, 60, 20261210, &s);
  std::vector<Isometry3F64> poses(s->n_cam);
  for (int j = 0; j < s->n_cam; ++j)
    for (int k = 0; k < 7; ++k) poses[j].params[k] = s->poses[7 * j + k];
  std::vector<VecF64_3> pts(s->n_pt);
  for (int i = 0; i < s->n_pt; ++i)
    for (int k = 0; k < 3; ++k) pts[i][k] = s->points[3 * i + k];
  std::vector<PinholeCameraReprojectionCostTerm> obs;
  for (int64_t o = 0; o < s->n_obs; ++o)
    obs.push_back({{s->obs_uv[2 * o], s->obs_uv[2 * o + 1]},
                   {0, static_cast<size_t>(s->obs_cam[o]), static_cast<size_t>(s->obs_pt[o])}});
  PinholeCameraF64 cam{{s->intrinsics[0], s->intrinsics[1], s->intrinsics[2], s->intrinsics[3]}, {640, 480}};
  auto vars = VarBuilder::new_()
                  .add_family("cams", VarFamily<PinholeCameraF64>::new_(VarKind::Conditioned, {cam}))
                  .add_family("poses", VarFamily<Isometry3F64>::new_with_const_ids(VarKind::Free, poses, {0}))
                  .add_family("points", VarFamily<VecF64_3>::new_(VarKind::Marginalized, pts))
                  .build();
  OptParams params;
  params.num_iterations = 3;
  params.initial_lm_damping = 1e-4;
  params.function_tolerance = 0.0;
  params.gradient_tolerance = 0.0;
  params.parameter_tolerance = 0.0;
  params.solver = LinearSolverEnum::SchurBlockSparseLdlt;
  auto cf = CostFn::new_boxed_robust(CostTerms::new_({"cams", "poses", "points"}, obs), HuberKernel::new_(1.0));
  auto sol = optimize_nlls(vars, {cf}, {}, params, 0);
  Optimizer opt(vars, {cf}, params, 0);
  for (int k = 0; k < 3; ++k) {
    auto info = opt.step();
    EXPECT(info.merit == sol.steps[k].merit, "step " + std::to_string(k) + " merit differs");
  }
  auto sol2 = opt.build_solution();
  EXPECT(sol2.final_cost == sol.final_cost, "final cost differs");
  std::printf("OK stepper_matches_optimize (%.9e)\n", sol.final_cost);
  sgba_synth_free(s);
}

int main() {
  simple_cam_marg_points();
  ba_converges();
  solver_validation();
  stepper_matches_optimize();
  if (g_fail) {
    std::printf("%d failure(s)\n", g_fail);
    return 1;
  }
  std::printf("all passed\n");
  return 0;
}

// sophus_opt.hpp -- header-only C++17 mirror of the sophus_opt API surface for
// the Schur-LM bundle-adjustment path, over the C ABI in sgba.h.
//
// Names, defaults and errors follow the reference crate:
//   optimize_nlls            crates/sophus_opt/src/nlls.rs:73-83
//   Optimizer                crates/sophus_opt/src/nlls/optimizer.rs:71-120,345-376,609-646
//   OptParams                crates/sophus_opt/src/nlls/optimizer_types.rs:161-240
//   StepInfo, TerminationReason  crates/sophus_opt/src/nlls/optimizer_types.rs:67-122
//   VarKind, VarFamily, VarBuilder  crates/sophus_opt/src/variables*.rs
//   CostTerms, CostFn        crates/sophus_opt/src/nlls/cost/cost_term.rs:98, cost/cost_fn.rs:127-152
//   HuberKernel              crates/sophus_opt/src/robust_kernel.rs
//   PinholeCameraReprojectionCostTerm
//                            crates/sophus_opt/src/nlls/functor_library/costs/pinhole_reprojection.rs:28-95
// Only the bundle-adjustment configuration runs on the GPU backend; anything
// else throws NotOnGpuPath.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <map>
#include <memory>
#include <optional>
#include <set>
#include <stdexcept>
#include <string>
#include <variant>
#include <vector>

#include "sgba.h"

namespace sgba {
namespace opt {

// ---- errors (NllsError, crates/sophus_opt/src/nlls/optimizer_types.rs:422-504) ----
struct NllsError : std::runtime_error {
  explicit NllsError(const std::string& m) : std::runtime_error(m) {}
};
struct SchurMissingFreeOrMarg : NllsError {
  using NllsError::NllsError;
};
struct SchurCostConnectsTwoMargFamilies : NllsError {
  using NllsError::NllsError;
};
struct NotOnGpuPath : NllsError {
  using NllsError::NllsError;
};
struct BackendError : NllsError {
  int status;
  BackendError(int s, const std::string& m) : NllsError(m), status(s) {}
};

inline void check(int status) {
  if (status == SGBA_OK) return;
  char buf[512];
  sgba_last_error(buf, sizeof(buf));
  if (status == SGBA_ERR_SCHUR_MISSING_FREE_OR_MARG) throw SchurMissingFreeOrMarg(buf);
  throw BackendError(status, buf);
}

// ---- variables ----
enum class VarKind { Free, Conditioned, Marginalized };

struct Isometry3F64 {
  std::array<double, 7> params{1, 0, 0, 0, 0, 0, 0};  // qw qx qy qz tx ty tz
  static Isometry3F64 identity() { return {}; }
  static Isometry3F64 from_params(const std::array<double, 7>& p) {
    const double n = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2] + p[3] * p[3]);
    if (std::fabs(n - 1.0) > 1e-6) throw std::invalid_argument("Invalid parameters for Isometry3F64");
    Isometry3F64 r;
    r.params = p;
    if (r.params[0] < 0.0)
      for (int k = 0; k < 4; ++k) r.params[k] = -r.params[k];
    return r;
  }
  std::array<double, 3> translation() const { return {params[4], params[5], params[6]}; }
};

struct PinholeCameraF64 {
  std::array<double, 4> params{1, 1, 0, 0};  // fx fy cx cy
  std::array<int, 2> image_size{640, 480};
  static PinholeCameraF64 from_params_and_size(const std::array<double, 4>& p, std::array<int, 2> sz) {
    return PinholeCameraF64{p, sz};
  }
};

using VecF64_3 = std::array<double, 3>;

template <class T>
struct VarFamily {
  VarKind kind;
  std::vector<T> members;
  std::set<size_t> constant_ids;
  static VarFamily new_(VarKind k, std::vector<T> m) { return VarFamily{k, std::move(m), {}}; }
  static VarFamily new_with_const_ids(VarKind k, std::vector<T> m, std::set<size_t> ids) {
    return VarFamily{k, std::move(m), std::move(ids)};
  }
  size_t num_active() const { return members.size() - constant_ids.size(); }
};

using AnyFamily = std::variant<VarFamily<PinholeCameraF64>, VarFamily<Isometry3F64>, VarFamily<VecF64_3>>;

inline VarKind kind_of(const AnyFamily& f) {
  return std::visit([](const auto& x) { return x.kind; }, f);
}
inline size_t scalars_of(const AnyFamily& f) {
  struct V {
    size_t operator()(const VarFamily<PinholeCameraF64>& x) const { return 4 * x.num_active(); }
    size_t operator()(const VarFamily<Isometry3F64>& x) const { return 6 * x.num_active(); }
    size_t operator()(const VarFamily<VecF64_3>& x) const { return 3 * x.num_active(); }
  };
  return std::visit(V{}, f);
}

struct VarFamilies {
  std::map<std::string, AnyFamily> collection;  // ordered by name, as the reference's BTreeMap
  template <class T>
  const std::vector<T>& get_members(const std::string& name) const {
    return std::get<VarFamily<T>>(collection.at(name)).members;
  }
  size_t num_free_scalars() const {
    size_t n = 0;
    for (const auto& kv : collection)
      if (kind_of(kv.second) == VarKind::Free) n += scalars_of(kv.second);
    return n;
  }
  size_t num_marg_scalars() const {
    size_t n = 0;
    for (const auto& kv : collection)
      if (kind_of(kv.second) == VarKind::Marginalized) n += scalars_of(kv.second);
    return n;
  }
};

struct VarBuilder {
  std::map<std::string, AnyFamily> families;
  static VarBuilder new_() { return {}; }
  template <class T>
  VarBuilder& add_family(const std::string& name, VarFamily<T> f) {
    families.insert_or_assign(name, AnyFamily(std::move(f)));
    return *this;
  }
  VarFamilies build() const { return VarFamilies{families}; }
};

// ---- costs ----
struct PinholeCameraReprojectionCostTerm {
  std::array<double, 2> uv_in_image;
  std::array<size_t, 3> entity_indices;  // intrinsics, pose, point
};

struct CostTerms {
  std::array<std::string, 3> family_names;
  std::vector<PinholeCameraReprojectionCostTerm> terms;
  static CostTerms new_(std::array<std::string, 3> names, std::vector<PinholeCameraReprojectionCostTerm> t) {
    return CostTerms{std::move(names), std::move(t)};
  }
};

struct HuberKernel {
  double delta;
  static HuberKernel new_(double d) { return HuberKernel{d}; }
};

struct CostFn {
  CostTerms cost_terms;
  std::optional<HuberKernel> robust_kernel;
  static CostFn new_boxed(CostTerms t) { return CostFn{std::move(t), std::nullopt}; }
  static CostFn new_boxed_robust(CostTerms t, HuberKernel k) { return CostFn{std::move(t), k}; }
};

// ---- params / results ----
enum class LinearSolverEnum {
  DenseLdlt, DenseLu, SparseLdlt, BlockSparseLdlt, FaerSparseQr, FaerSparseLu, FaerSparseLdlt,
  FaerSparseLblt, SchurBlockSparseLdlt, SchurSparseLdlt, SchurFaerSparseLdlt,
};
inline bool is_schur(LinearSolverEnum s) {
  return s == LinearSolverEnum::SchurBlockSparseLdlt || s == LinearSolverEnum::SchurSparseLdlt ||
         s == LinearSolverEnum::SchurFaerSparseLdlt;
}

struct OptParams {
  size_t num_iterations = 100;
  double initial_lm_damping = 10.0;
  bool parallelize = true;
  LinearSolverEnum solver = LinearSolverEnum::FaerSparseLdlt;
  bool skip_final_hessian = false;
  double function_tolerance = 1e-10;
  double gradient_tolerance = 1e-14;
  double parameter_tolerance = 1e-12;
  size_t max_consecutive_rejects = 20;
};

enum class TerminationReason { FunctionTolerance = 1, GradientTolerance, ParameterTolerance, MaxIterations,
                               MaxConsecutiveRejects };

struct StepInfo {
  double merit, smooth_cost;
  bool did_outer_step;
  size_t inner_step;
  double lm_damping;
  bool in_phase1;
  std::optional<TerminationReason> termination;
  double new_merit, gain_ratio, max_step;
  bool accepted;
};

// A block of the covariance or of the precision matrix, row-major.
struct Block {
  int rows = 0, cols = 0;
  std::vector<double> values;
};

// OptimizationSolution (crates/sophus_opt/src/nlls/optimizer_types.rs:242-370).
// covariance_block / precision_block answer from the final Hessian on the
// GPU; the device problem stays with the solution and the covariance is
// prepared on the first query (the reference builds its Covariance lazily).
struct OptimizationSolution {
  VarFamilies variables;
  double final_cost;
  std::vector<StepInfo> steps;
  std::shared_ptr<sgba_problem> problem{};
  std::array<std::string, 3> names{};  // camera, pose and point families
  std::shared_ptr<bool> cov_ready = std::make_shared<bool>(false);

  // Sigma(i, j), or nullopt for a constant variable or another family.
  std::optional<Block> covariance_block(const std::string& row_family, size_t row_idx, const std::string& col_family,
                                        size_t col_idx) const {
    return query(SGBA_QUERY_COVARIANCE, row_family, row_idx, col_family, col_idx);
  }
  // H(i, j) of the undamped final Hessian, or nullopt.
  std::optional<Block> precision_block(const std::string& row_family, size_t row_idx, const std::string& col_family,
                                       size_t col_idx) const {
    return query(SGBA_QUERY_PRECISION, row_family, row_idx, col_family, col_idx);
  }
  std::optional<Block> query(int mode, const std::string& rf, size_t ri, const std::string& cf, size_t ci) const {
    if (!problem) throw NllsError("this solution holds no final Hessian");
    auto kind = [this](const std::string& f) {
      return f == names[0] ? SGBA_VAR_INTRINSICS : f == names[1] ? SGBA_VAR_POSE : f == names[2] ? SGBA_VAR_POINT : -1;
    };
    const int rk = kind(rf), ck = kind(cf);
    if (rk < 0 || ck < 0) return std::nullopt;
    if (!*cov_ready) {
      check(sgba_covariance_prepare(problem.get(), nullptr));
      *cov_ready = true;
    }
    sgba_cov_query q{rk, static_cast<int32_t>(ri), ck, static_cast<int32_t>(ci)};
    Block b;
    b.values.assign(36, 0.0);
    int32_t dims[2] = {0, 0};
    check(sgba_covariance_blocks(problem.get(), mode, 1, &q, b.values.data(), dims));
    if (dims[0] <= 0) return std::nullopt;
    b.rows = dims[0];
    b.cols = dims[1];
    b.values.resize(static_cast<size_t>(b.rows) * b.cols);
    return b;
  }
};

namespace detail {

struct Flat {
  std::vector<double> poses, points, uv;
  std::vector<uint8_t> pconst, qconst;
  std::vector<int32_t> ocam, opt;
  std::array<double, 4> intr{};
  double huber = 0.0;
  std::array<std::string, 3> names;
};

// validate_solver_config (crates/sophus_opt/src/nlls/optimizer.rs:649-717)
inline void validate(const VarFamilies& v, const std::vector<CostFn>& costs, const OptParams& p) {
  if (!is_schur(p.solver)) throw NotOnGpuPath("the GPU path needs a Schur solver");
  if (v.num_free_scalars() == 0 || v.num_marg_scalars() == 0)
    throw SchurMissingFreeOrMarg("Schur solver needs free and marginalized variables");
  for (const auto& c : costs) {
    int marg = 0;
    for (const auto& n : c.cost_terms.family_names) {
      auto it = v.collection.find(n);
      if (it != v.collection.end() && kind_of(it->second) == VarKind::Marginalized) ++marg;
    }
    if (marg > 1) throw SchurCostConnectsTwoMargFamilies("cost connects two marginalized families");
  }
}

inline Flat flatten(const VarFamilies& v, const std::vector<CostFn>& costs) {
  if (costs.size() != 1) throw NotOnGpuPath("exactly one reprojection CostFn runs on the GPU path");
  const CostFn& c = costs[0];
  Flat f;
  f.names = c.cost_terms.family_names;
  const auto* cams = std::get_if<VarFamily<PinholeCameraF64>>(&v.collection.at(f.names[0]));
  const auto* poses = std::get_if<VarFamily<Isometry3F64>>(&v.collection.at(f.names[1]));
  const auto* pts = std::get_if<VarFamily<VecF64_3>>(&v.collection.at(f.names[2]));
  if (!cams || !poses || !pts) throw NotOnGpuPath("families must be (PinholeCameraF64, Isometry3F64, VecF64<3>)");
  if (cams->kind != VarKind::Conditioned || poses->kind != VarKind::Free || pts->kind != VarKind::Marginalized)
    throw NotOnGpuPath("kinds must be (Conditioned, Free, Marginalized)");
  if (cams->members.size() != 1) throw NotOnGpuPath("one intrinsics member is supported");
  f.intr = cams->members[0].params;
  for (const auto& m : poses->members) f.poses.insert(f.poses.end(), m.params.begin(), m.params.end());
  f.pconst.assign(poses->members.size(), 0);
  for (size_t i : poses->constant_ids) f.pconst.at(i) = 1;
  for (const auto& m : pts->members) f.points.insert(f.points.end(), m.begin(), m.end());
  f.qconst.assign(pts->members.size(), 0);
  for (size_t i : pts->constant_ids) f.qconst.at(i) = 1;
  for (const auto& t : c.cost_terms.terms) {
    if (t.entity_indices[0] != 0) throw NotOnGpuPath("intrinsics index must be 0");
    f.ocam.push_back(static_cast<int32_t>(t.entity_indices[1]));
    f.opt.push_back(static_cast<int32_t>(t.entity_indices[2]));
    f.uv.push_back(t.uv_in_image[0]);
    f.uv.push_back(t.uv_in_image[1]);
  }
  f.huber = c.robust_kernel ? c.robust_kernel->delta : 0.0;
  return f;
}

inline sgba_problem* create(const Flat& f, int device) {
  sgba_problem_desc d{};
  d.n_cam = static_cast<int32_t>(f.pconst.size());
  d.poses = f.poses.data();
  d.pose_const = f.pconst.data();
  d.n_pt = static_cast<int32_t>(f.qconst.size());
  d.points = f.points.data();
  d.point_const = f.qconst.data();
  for (int k = 0; k < 4; ++k) d.intrinsics[k] = f.intr[k];
  d.n_obs = static_cast<int64_t>(f.ocam.size());
  d.obs_cam = f.ocam.data();
  d.obs_pt = f.opt.data();
  d.obs_uv = f.uv.data();
  d.huber_delta = f.huber;
  sgba_problem* p = nullptr;
  check(sgba_problem_create(&d, device, &p));
  return p;
}

inline sgba_opt_params cparams(const OptParams& p) {
  sgba_opt_params c{};
  c.num_iterations = static_cast<int32_t>(p.num_iterations);
  c.initial_lm_damping = p.initial_lm_damping;
  c.function_tolerance = p.function_tolerance;
  c.gradient_tolerance = p.gradient_tolerance;
  c.parameter_tolerance = p.parameter_tolerance;
  c.max_consecutive_rejects = p.max_consecutive_rejects > (size_t(1) << 62)
                                  ? (int64_t(1) << 62)
                                  : static_cast<int64_t>(p.max_consecutive_rejects);
  c.skip_final_hessian = p.skip_final_hessian ? 1 : 0;
  return c;
}

inline StepInfo step_info(const sgba_iter_record& r, size_t k) {
  StepInfo s{};
  s.merit = r.merit;
  s.smooth_cost = r.merit;
  s.did_outer_step = false;
  s.inner_step = k;
  s.lm_damping = r.lm_damping;
  s.in_phase1 = false;
  if (r.termination != SGBA_TERM_NONE) s.termination = static_cast<TerminationReason>(r.termination);
  s.new_merit = r.new_merit;
  s.gain_ratio = r.gain_ratio;
  s.max_step = r.max_step;
  s.accepted = r.accepted != 0;
  return s;
}

inline VarFamilies write_back(const VarFamilies& v, const Flat& f, const std::vector<double>& poses,
                              const std::vector<double>& points) {
  VarFamilies out = v;
  auto& pf = std::get<VarFamily<Isometry3F64>>(out.collection.at(f.names[1]));
  for (size_t i = 0; i < pf.members.size(); ++i)
    for (int k = 0; k < 7; ++k) pf.members[i].params[k] = poses[7 * i + k];
  auto& qf = std::get<VarFamily<VecF64_3>>(out.collection.at(f.names[2]));
  for (size_t i = 0; i < qf.members.size(); ++i)
    for (int k = 0; k < 3; ++k) qf.members[i][k] = points[3 * i + k];
  return out;
}

}  // namespace detail

// Stateful optimizer (Optimizer::new / step / build_solution).
class Optimizer {
 public:
  Optimizer(VarFamilies variables, std::vector<CostFn> costs, OptParams params, int device = -1)
      : vars_(std::move(variables)), params_(params) {
    detail::validate(vars_, costs, params_);
    flat_ = detail::flatten(vars_, costs);
    p_ = std::shared_ptr<sgba_problem>(detail::create(flat_, device), sgba_problem_destroy);
    sgba_opt_params c = detail::cparams(params_);
    check(sgba_optimizer_init(p_.get(), &c));
  }
  Optimizer(const Optimizer&) = delete;
  Optimizer& operator=(const Optimizer&) = delete;
  StepInfo step() {
    sgba_iter_record r{};
    check(sgba_optimizer_step(p_.get(), &r));
    steps_.push_back(detail::step_info(r, steps_.size()));
    return steps_.back();
  }
  // The solution shares the device problem (its covariance is prepared at the
  // variables of its first query; the reference's build_solution consumes
  // the optimizer, so no step comes between).
  OptimizationSolution build_solution() {
    std::vector<double> poses(flat_.poses.size()), points(flat_.points.size());
    check(sgba_get_variables(p_.get(), poses.data(), points.data()));
    double cost = 0.0;
    check(sgba_get_cost(p_.get(), &cost));
    return OptimizationSolution{detail::write_back(vars_, flat_, poses, points), cost, steps_, p_, flat_.names};
  }

 private:
  VarFamilies vars_;
  OptParams params_;
  detail::Flat flat_;
  std::shared_ptr<sgba_problem> p_;
  std::vector<StepInfo> steps_;
};

// optimize_nlls: step until a termination reason, then build_solution.
inline OptimizationSolution optimize_nlls(const VarFamilies& variables, const std::vector<CostFn>& cost_fns,
                                          const std::vector<CostFn>& eq_fns, const OptParams& params,
                                          int device = -1) {
  if (!eq_fns.empty()) throw NotOnGpuPath("equality constraints are outside the GPU path");
  detail::validate(variables, cost_fns, params);
  detail::Flat f = detail::flatten(variables, cost_fns);
  sgba_problem* p = detail::create(f, device);
  sgba_opt_params c = detail::cparams(params);
  const int cap = static_cast<int>(params.num_iterations > 0 ? params.num_iterations : 1);
  std::vector<sgba_iter_record> recs(cap);
  int32_t n = 0, term = 0;
  int st = sgba_optimize(p, &c, recs.data(), cap, &n, &term);
  std::vector<double> poses(f.poses.size()), points(f.points.size());
  double cost = 0.0;
  if (st == SGBA_OK) st = sgba_get_variables(p, poses.data(), points.data());
  if (st == SGBA_OK) st = sgba_get_cost(p, &cost);
  if (st != SGBA_OK) {
    sgba_problem_destroy(p);
    check(st);
  }
  std::vector<StepInfo> steps;
  for (int k = 0; k < n && k < cap; ++k) steps.push_back(detail::step_info(recs[k], k));
  // the device problem stays with the solution (covariance / precision queries)
  return OptimizationSolution{detail::write_back(variables, f, poses, points), cost, steps,
                              std::shared_ptr<sgba_problem>(p, sgba_problem_destroy), f.names};
}

}  // namespace opt
}  // namespace sgba

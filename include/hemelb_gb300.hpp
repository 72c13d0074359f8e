// hemelb_gb300.hpp -- C++ RAII wrapper over the C ABI (header only, no HemeLB
// dependency).  Status codes become exceptions, as HemeLB reports failures with
// hemelb::Exception (Code/Exception.h); the solver owns its device memory.
#ifndef HEMELB_GB300_HPP
#define HEMELB_GB300_HPP

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "hemelb_gb300.h"

namespace hemelb_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc, const hlbg_ctx* ctx, const char* what) {
  if (rc != HLBG_OK) {
    std::string msg = std::string(what) + " failed (" + std::to_string(rc) + ")";
    if (ctx) msg += ": " + std::string(hlbg_last_error(ctx));
    throw Error(rc, msg);
  }
}

/// A sparse block geometry owned by the caller, built site by site in the
/// reference's terms (global coordinates, SiteData wall/iolet bit masks, iolet
/// id, site type, cut distances).
class GeometryBuilder {
 public:
  explicit GeometryBuilder(int q = 19) : q_(q) {}

  void AddFluidSite(int64_t x, int64_t y, int64_t z, uint32_t wall_mask = 0, uint32_t iolet_mask = 0,
                    int32_t iolet_id = -1, int8_t site_type = HLBG_SITE_FLUID,
                    const double* cut_distances = nullptr) {
    sites_.push_back({x, y, z, wall_mask, iolet_mask, iolet_id, site_type});
    for (int k = 0; k < q_ - 1; ++k)
      cuts_.push_back(cut_distances ? (float)cut_distances[k] : -1.0f);
    for (int a = 0; a < 3; ++a) {
      int64_t c = a == 0 ? x : (a == 1 ? y : z);
      if (c < 0) throw Error(HLBG_ERR_INVAL, "negative site coordinate");
      if (c / 8 + 1 > nb_[a]) nb_[a] = (int32_t)(c / 8 + 1);
    }
  }

  /// Finalise into the C view; the builder must outlive the view's use.
  const hlbg_geometry& View() {
    blocks_.clear();
    block_index_.assign((size_t)nb_[0] * nb_[1] * nb_[2], -1);
    masks_.clear();
    link_site_.clear();
    wall_.clear();
    iolet_.clear();
    ioid_.clear();
    stype_.clear();
    rec_cuts_.clear();
    std::vector<std::pair<int64_t, size_t>> order;
    for (size_t i = 0; i < sites_.size(); ++i) {
      const Site& s = sites_[i];
      size_t bi = ((size_t)(s.x / 8) * nb_[1] + s.y / 8) * nb_[2] + s.z / 8;
      if (block_index_[bi] < 0) {
        block_index_[bi] = (int64_t)blocks_.size() / 3;
        blocks_.push_back((int32_t)(s.x / 8));
        blocks_.push_back((int32_t)(s.y / 8));
        blocks_.push_back((int32_t)(s.z / 8));
        for (int w = 0; w < 8; ++w) masks_.push_back(0);
      }
      int64_t b = block_index_[bi];
      int l = (int)(((s.x % 8) * 8 + s.y % 8) * 8 + s.z % 8);
      masks_[b * 8 + l / 64] |= 1ull << (l % 64);
      if (s.wall || s.iolet) order.push_back({b * 512 + l, i});
    }
    std::sort(order.begin(), order.end());
    for (auto& [slot, i] : order) {
      const Site& s = sites_[i];
      link_site_.push_back(slot);
      wall_.push_back(s.wall);
      iolet_.push_back(s.iolet);
      ioid_.push_back(s.ioid);
      stype_.push_back(s.type);
      for (int k = 0; k < q_ - 1; ++k) rec_cuts_.push_back(cuts_[i * (q_ - 1) + k]);
    }
    view_ = hlbg_geometry{};
    view_.q = q_;
    view_.block_size = 8;
    for (int a = 0; a < 3; ++a) view_.blocks[a] = nb_[a];
    view_.n_blocks = (int64_t)blocks_.size() / 3;
    view_.block_coords = blocks_.data();
    view_.fluid_mask = masks_.data();
    view_.n_link_sites = (int64_t)link_site_.size();
    view_.link_site = link_site_.data();
    view_.wall_mask = wall_.data();
    view_.iolet_mask = iolet_.data();
    view_.iolet_id = ioid_.data();
    view_.site_type = stype_.data();
    view_.cut_distance = rec_cuts_.data();
    return view_;
  }

 private:
  struct Site {
    int64_t x, y, z;
    uint32_t wall, iolet;
    int32_t ioid;
    int8_t type;
  };
  int q_;
  int32_t nb_[3] = {0, 0, 0};
  std::vector<Site> sites_;
  std::vector<float> cuts_;
  std::vector<int32_t> blocks_;
  std::vector<int64_t> block_index_;
  std::vector<uint64_t> masks_;
  std::vector<int64_t> link_site_;
  std::vector<uint32_t> wall_, iolet_;
  std::vector<int32_t> ioid_;
  std::vector<int8_t> stype_;
  std::vector<float> rec_cuts_;
  hlbg_geometry view_{};
};

/// Owns one device context: the distributions, the site layout and the iolets.
class Solver {
 public:
  Solver(const hlbg_geometry& g, const hlbg_params& p, const std::vector<hlbg_iolet>& inlets,
         const std::vector<hlbg_iolet>& outlets) {
    n_iolets_ = inlets.size() + outlets.size();
    int rc = hlbg_create(&g, &p, inlets.data(), (int32_t)inlets.size(), outlets.data(),
                         (int32_t)outlets.size(), &ctx_);
    if (rc != HLBG_OK) {
      std::string msg = ctx_ ? hlbg_last_error(ctx_) : "";
      hlbg_destroy(ctx_);
      ctx_ = nullptr;
      throw Error(rc, "hlbg_create failed: " + msg);
    }
  }
  ~Solver() { hlbg_destroy(ctx_); }
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  hlbg_ctx* get() const { return ctx_; }
  int64_t SiteCount() const { return hlbg_site_count(ctx_); }

  void SetEquilibrium(double rho = 1.0, double ux = 0.0, double uy = 0.0, double uz = 0.0) {
    check(hlbg_init_equilibrium(ctx_, rho, ux, uy, uz), ctx_, "hlbg_init_equilibrium");
  }
  void Step(int n = 1) {
    check(hlbg_step(ctx_, n, nullptr), ctx_, "hlbg_step");
    check(hlbg_sync(ctx_), ctx_, "hlbg_sync");
  }
  void StreamAndCollide(int64_t first, int64_t count) {
    check(hlbg_stream_and_collide_range(ctx_, first, count), ctx_, "hlbg_stream_and_collide_range");
  }
  void PostStep(int64_t first, int64_t count) {
    check(hlbg_post_step_range(ctx_, first, count), ctx_, "hlbg_post_step_range");
  }
  void SwapOldAndNew() { check(hlbg_swap(ctx_), ctx_, "hlbg_swap"); }
  void GetF(double* host, int which) { check(hlbg_get_f(ctx_, host, which), ctx_, "hlbg_get_f"); }
  void PutF(const double* host, int which) { check(hlbg_put_f(ctx_, host, which), ctx_, "hlbg_put_f"); }
  hlbg_stats Reduce() {
    hlbg_stats st{};
    int rc = hlbg_reduce(ctx_, &st);
    if (rc != HLBG_OK && rc != HLBG_ERR_UNSTABLE) check(rc, ctx_, "hlbg_reduce");
    return st;
  }
  /// n steps with the StabilityTester fused in; the stats of the step before the last.
  hlbg_stats StepMonitored(int n = 1) {
    hlbg_stats st{};
    int rc = hlbg_step_monitored(ctx_, n, &st);
    if (rc != HLBG_OK && rc != HLBG_ERR_UNSTABLE) check(rc, ctx_, "hlbg_step_monitored");
    return st;
  }
  struct Steady {
    int64_t steps_to_steady, steps_run;
    double final_rel_du;
    int status;  // HLBG_OK, HLBG_ERR_TIMEOUT or HLBG_ERR_UNSTABLE
  };
  Steady RunToSteady(double tol, double u_ref, int64_t max_steps, int32_t check_batch = 25) {
    Steady r{};
    r.status = hlbg_run_to_steady(ctx_, tol, u_ref, max_steps, check_batch, &r.steps_to_steady, &r.steps_run,
                                  &r.final_rel_du);
    if (r.status != HLBG_OK && r.status != HLBG_ERR_TIMEOUT && r.status != HLBG_ERR_UNSTABLE)
      check(r.status, ctx_, "hlbg_run_to_steady");
    return r;
  }
  void SetTimeStep(uint64_t t1) { check(hlbg_set_time_step(ctx_, t1), ctx_, "hlbg_set_time_step"); }
  void SetIolets(const std::vector<hlbg_iolet>& inlets, const std::vector<hlbg_iolet>& outlets) {
    check(hlbg_set_iolets(ctx_, inlets.data(), (int32_t)inlets.size(), outlets.data(), (int32_t)outlets.size()),
          ctx_, "hlbg_set_iolets");
  }
  void GetMacro(double* rho, double* u) { check(hlbg_get_macro(ctx_, rho, u), ctx_, "hlbg_get_macro"); }
  std::vector<double> IoletFlux() {
    std::vector<double> out(n_iolets_);
    check(hlbg_iolet_flux(ctx_, out.data(), (int32_t)out.size()), ctx_, "hlbg_iolet_flux");
    return out;
  }
  std::vector<double> WallShearStress() {
    std::vector<double> out((size_t)SiteCount());
    check(hlbg_wall_shear_stress(ctx_, out.data()), ctx_, "hlbg_wall_shear_stress");
    return out;
  }
  hlbg_incomp Incompressibility() {
    hlbg_incomp r{};
    check(hlbg_incompressibility(ctx_, &r), ctx_, "hlbg_incompressibility");
    return r;
  }
  void WriteCheckpoint(const std::string& path, uint64_t timestep, double voxel_size = 1.0,
                       const double* origin = nullptr, bool append = false) {
    const double zero[3] = {0.0, 0.0, 0.0};
    check(hlbg_write_checkpoint(ctx_, path.c_str(), timestep, voxel_size, origin ? origin : zero, append ? 1 : 0),
          ctx_, "hlbg_write_checkpoint");
  }
  /// Loads the record of `timestep` (the last one when negative); returns its timestep.
  uint64_t ReadCheckpoint(const std::string& path, int64_t timestep = -1) {
    uint64_t found = 0;
    check(hlbg_read_checkpoint(ctx_, path.c_str(), timestep, &found), ctx_, "hlbg_read_checkpoint");
    return found;
  }
  int32_t Autotune(int32_t steps_per_trial = 3) {
    int32_t v = 0;
    float ms = 0.f;
    check(hlbg_autotune(ctx_, steps_per_trial, &v, &ms), ctx_, "hlbg_autotune");
    return v;
  }

 private:
  hlbg_ctx* ctx_ = nullptr;
  size_t n_iolets_ = 0;
};

}  // namespace hemelb_gb300

#endif

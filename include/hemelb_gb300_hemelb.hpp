// hemelb_gb300_hemelb.hpp -- HemeLB-side plugin over the C ABI.
//
// Include from inside a HemeLB build (it uses HemeLB's own types).  Two ways in:
//
//  * GpuStreamer<Collision>: a type satisfying lb::streamer (Code/lb/concepts.h:91-102),
//    usable as any of the six Traits streamers (Code/Traits.h:17-39).  Its
//    StreamAndCollide / PostStep run the range on the device; the host FieldData
//    stays the source of truth, so every step uploads fOld/fNew once and every
//    PostStep downloads fNew.  This is the compatibility mode.
//
//  * GpuLBM: the whole-step replacement of lb::LBM's IteratedAction phases
//    (Code/lb/lb.hpp:162-309).  The distributions stay on the device; PreReceive
//    runs one full update (StreamAndCollide over all six ranges, PostStep, swap);
//    SyncToHost() fills the FieldData when property output or a checkpoint needs it.
//
// Both read the Domain through the same accessors the reference streamers use
// (Site::HasWall / HasIolet / GetIoletId / GetSiteType / GetWallDistance /
// GetGlobalSiteCoords) and hand the device a sparse block geometry built from them.
#ifndef HEMELB_GB300_HEMELB_HPP
#define HEMELB_GB300_HEMELB_HPP

#include <map>
#include <memory>
#include <vector>

#include "hemelb_gb300.hpp"

namespace hemelb_gb300 {

inline hlbg_iolet ToCIolet(const hemelb::lb::InOutLet& io) {
  hlbg_iolet c{};
  auto pos = io.GetPosition();
  auto n = io.GetNormal();
  for (int k = 0; k < 3; ++k) {
    c.position[k] = pos[k];
    c.normal[k] = n[k];
  }
  if (auto* cos = dynamic_cast<const hemelb::lb::InOutLetCosine*>(&io)) {
    c.model = HLBG_IOLET_COSINE;
    c.density_mean = cos->GetDensityMean();
    c.density_amp = cos->GetDensityAmp();
    c.phase = cos->GetPhase();
    c.period = cos->GetPeriod();
  } else if (auto* par = dynamic_cast<const hemelb::lb::InOutLetParabolicVelocity*>(&io)) {
    c.model = HLBG_IOLET_PARABOLIC;
    c.radius = par->GetRadius();
    c.max_speed = par->GetMaxSpeed();
  } else {
    throw Error(HLBG_ERR_INVAL, "iolet type without a device model");
  }
  return c;
}

/// Build the device geometry from a reference Domain (one rank, all sites local).
template <class Lattice, class FieldDataT>
GeometryBuilder FromFieldData(FieldDataT& fd) {
  GeometryBuilder gb(Lattice::NUMVECTORS);
  auto& dom = fd.GetDomain();
  const hemelb::site_t n = dom.GetLocalFluidSiteCount();
  std::vector<double> cuts(Lattice::NUMVECTORS - 1);
  for (hemelb::site_t i = 0; i < n; ++i) {
    auto site = fd.GetSite(i);
    uint32_t wm = 0, im = 0;
    for (unsigned d = 1; d < Lattice::NUMVECTORS; ++d) {
      if (site.HasWall(d)) wm |= 1u << (d - 1);
      if (site.HasIolet(d)) im |= 1u << (d - 1);
      cuts[d - 1] = site.template GetWallDistance<Lattice>(d);
    }
    const auto& x = site.GetGlobalSiteCoords();
    gb.AddFluidSite(x[0], x[1], x[2], wm, im, site.GetIoletId(), (int8_t)site.GetSiteType(),
                    cuts.data());
  }
  return gb;
}

/// Physics of the device update (the Traits selection, Code/Traits.h:17-39, and
/// the iolet values of the two BoundaryValues objects).
struct DeviceConfig {
  int kernel = HLBG_KERNEL_LBGK;
  int wall = HLBG_WALL_SBB;
  int inlet = HLBG_IOLET_NASH;
  int outlet = HLBG_IOLET_NASH;
  int precision = HLBG_FP64;
  std::vector<hlbg_iolet> inlets, outlets;
};

inline DeviceConfig MakeConfig(int kernel, int wall, int inlet, int outlet,
                               hemelb::lb::BoundaryValues& in, hemelb::lb::BoundaryValues& out,
                               int precision = HLBG_FP64) {
  DeviceConfig c;
  c.kernel = kernel;
  c.wall = wall;
  c.inlet = inlet;
  c.outlet = outlet;
  c.precision = precision;
  for (unsigned i = 0; i < in.GetLocalIoletCount(); ++i) c.inlets.push_back(ToCIolet(*in.GetLocalIolet(i)));
  for (unsigned i = 0; i < out.GetLocalIoletCount(); ++i) c.outlets.push_back(ToCIolet(*out.GetLocalIolet(i)));
  return c;
}

/// One device context per FieldData, shared by the six streamers of an LBM.
struct DeviceField {
  GeometryBuilder geometry;
  std::unique_ptr<Solver> solver;
  const double* uploaded_fold = nullptr;  // host fOld buffer at the last upload
};

template <class FieldDataT>
inline std::map<const FieldDataT*, std::shared_ptr<DeviceField>>& Registry() {
  static std::map<const FieldDataT*, std::shared_ptr<DeviceField>> r;
  return r;
}

/// Create the device context for a FieldData; call once, where SimBuilder calls
/// LBM::Initialise (Code/configuration/SimBuilder.h:163-176).
template <class Lattice>
DeviceField& Attach(hemelb::geometry::FieldData& fd, const hemelb::lb::LbmParameters& p,
                    const DeviceConfig& cfg) {
  auto& slot = Registry<hemelb::geometry::FieldData>()[&fd];
  slot = std::make_shared<DeviceField>();
  slot->geometry = FromFieldData<Lattice>(fd);
  hlbg_params cp{};
  cp.kernel = cfg.kernel;
  cp.wall = cfg.wall;
  cp.inlet = cfg.inlet;
  cp.outlet = cfg.outlet;
  cp.precision = cfg.precision;
  cp.tau = p.GetTau();
  slot->solver = std::make_unique<Solver>(slot->geometry.View(), cp, cfg.inlets, cfg.outlets);
  return *slot;
}

inline DeviceField& Attached(const hemelb::geometry::FieldData& fd) {
  auto& reg = Registry<hemelb::geometry::FieldData>();
  auto it = reg.find(&fd);
  if (it == reg.end() || !it->second) throw Error(HLBG_ERR_STATE, "FieldData has no device context (Attach first)");
  return *it->second;
}

/// Satisfies lb::streamer: runs its range on the device, host FieldData stays the
/// source of truth (upload once per step, fNew downloaded after each PostStep).
template <class Collision>
class GpuStreamer {
 public:
  using CollisionType = Collision;
  using KernelType = typename Collision::KernelType;
  using LatticeType = typename Collision::LatticeType;
  using VarsType = typename Collision::VarsType;

  explicit GpuStreamer(hemelb::lb::InitParams& ip) : boundary_(ip.boundaryObject) {}

  void StreamAndCollide(const hemelb::site_t first, const hemelb::site_t count,
                        const hemelb::lb::LbmParameters*, hemelb::geometry::FieldData& fd,
                        hemelb::lb::MacroscopicPropertyCache&) {
    DeviceField& dev = Attached(fd);
    const double* fold = fd.GetFOld(0);
    if (dev.uploaded_fold != fold) {  // a new step: FieldData swapped its buffers
      dev.solver->PutF(fold, 0);
      dev.solver->PutF(fd.GetFNew(0), 1);
      dev.uploaded_fold = fold;
      if (boundary_) check(hlbg_set_time_step(dev.solver->get(), boundary_->GetTimeStep()),
                           dev.solver->get(), "hlbg_set_time_step");
    }
    dev.solver->StreamAndCollide(first, count);
  }

  void PostStep(const hemelb::site_t first, const hemelb::site_t count,
                const hemelb::lb::LbmParameters*, hemelb::geometry::FieldData& fd,
                hemelb::lb::MacroscopicPropertyCache&) {
    DeviceField& dev = Attached(fd);
    dev.solver->PostStep(first, count);
    dev.solver->GetF(fd.GetFNew(0), 1);
  }

 private:
  hemelb::lb::BoundaryValues* boundary_;
};

/// Whole-step replacement of lb::LBM's IteratedAction phases: the distributions
/// stay on the device; one hlbg_step per PreReceive.
class GpuLBM {
 public:
  GpuLBM(hemelb::geometry::FieldData& fd, DeviceField& dev) : fd_(fd), dev_(dev) {}
  void RequestComms() {}  // one rank: no halo (FieldData::SendAndReceive)
  void PreSend() {}       // no domain-edge sites on one rank
  void PreReceive() { dev_.solver->Step(1); }  // StreamAndCollide + PostStep + swap
  void PostReceive() {}
  void EndIteration() {}
  /// Fill the host FieldData (fOld, fNew) from the device.
  void SyncToHost() {
    dev_.solver->GetF(fd_.GetFOld(0), 0);
    dev_.solver->GetF(fd_.GetFNew(0), 1);
  }
  void SetInitialEquilibrium(double rho, double ux, double uy, double uz) {
    dev_.solver->SetEquilibrium(rho, ux, uy, uz);
  }
  hlbg_stats Stability() { return dev_.solver->Reduce(); }

 private:
  hemelb::geometry::FieldData& fd_;
  DeviceField& dev_;
};

}  // namespace hemelb_gb300

#endif

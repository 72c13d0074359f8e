// Driver that runs the REFERENCE's own LB streamer, collision, kernel, lattice and
// iolet code (compiled from the HemeLB sources) over a geometry prepared by the
// oracle, to pin the oracle's restatement.  Test infrastructure only.
//
// It mirrors lb::LBM's per-step order for one rank (Code/lb/lb.hpp:176-309):
// StreamAndCollide over the six collision-type ranges, PostStep over the same
// ranges, then FieldData::SwapOldAndNew and SimulationState::Increment
// (Code/SimulationMaster.impl.h:218-219).  The TRT kernel of this revision does
// not compile as it stands (Code/lb/kernels/TRT.h:42-54 and :62-92); the recipe in
// build_ref.py applies a build-time patch to those lines only, so the LBGK and the
// TRT kernels both run here from the reference's own source.
//
// Input / output: a little-endian binary file written by oracle/refbuild/run_ref.py.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "lb/iolets/BoundaryValues.h"
#include "lb/iolets/InOutLetCosine.h"
#include "lb/iolets/InOutLetParabolicVelocity.h"
#include "lb/lattices/D3Q15.h"
#include "lb/lattices/D3Q19.h"
#include "lb/kernels/LBGK.h"
#include "lb/kernels/TRT.h"
#include "lb/collisions/Normal.h"
#include "lb/streamers/BulkStreamer.h"
#include "lb/streamers/StreamerTypeFactory.h"
#include "lb/streamers/SimpleBounceBack.h"
#include "lb/streamers/BouzidiFirdaousLallemand.h"
#include "lb/streamers/NashZerothOrderPressure.h"
#include "lb/streamers/LaddIolet.h"

using namespace hemelb;

namespace {

struct Reader {
  FILE* f;
  template <class T>
  T get() {
    T v;
    if (fread(&v, sizeof(T), 1, f) != 1) {
      fprintf(stderr, "short read\n");
      exit(2);
    }
    return v;
  }
  template <class T>
  void arr(std::vector<T>& v, size_t n) {
    v.resize(n);
    if (n && fread(v.data(), sizeof(T), n, f) != n) {
      fprintf(stderr, "short read\n");
      exit(2);
    }
  }
};

struct IoletIn {
  int32_t model;
  double pos[3], normal[3], mean, amp, phase, period, radius, max_speed, vel_period;
  uint64_t warmup;
};

lb::InOutLet* make_iolet(const IoletIn& in) {
  if (in.model == 0) {
    auto* c = new lb::InOutLetCosine();
    c->SetDensityMean(in.mean);
    c->SetDensityAmp(in.amp);
    c->SetPhase(in.phase);
    c->SetPeriod(in.period);
    c->SetWarmup((unsigned)in.warmup);
    c->SetPosition(LatticePosition(in.pos[0], in.pos[1], in.pos[2]));
    c->SetNormal(util::Vector3D<Dimensionless>(in.normal[0], in.normal[1], in.normal[2]));
    return c;
  }
  auto* v = new lb::InOutLetParabolicVelocity();
  v->SetMaxSpeed(in.max_speed);
  v->SetWarmup((unsigned)in.warmup);
  v->SetRadius(in.radius);
  v->SetPosition(LatticePosition(in.pos[0], in.pos[1], in.pos[2]));
  v->SetNormal(util::Vector3D<Dimensionless>(in.normal[0], in.normal[1], in.normal[2]));
  return v;
}

template <class KERN, template <class> class WALL, template <class> class INL, template <class> class OUTL>
int run(geometry::FieldData& fd, const lb::LbmParameters& params, lb::BoundaryValues& inlets,
        lb::BoundaryValues& outlets, const site_t counts[6], lb::SimulationState& state, int nsteps,
        int mode) {
  using Coll = lb::Normal<KERN>;
  using Mid = lb::BulkStreamer<Coll>;
  using Wall = lb::StreamerTypeFactory<WALL<Coll>, lb::NullLink<Coll>>;
  using Inl = lb::StreamerTypeFactory<lb::NullLink<Coll>, INL<Coll>>;
  using Outl = lb::StreamerTypeFactory<lb::NullLink<Coll>, OUTL<Coll>>;
  using InlW = lb::StreamerTypeFactory<WALL<Coll>, INL<Coll>>;
  using OutlW = lb::StreamerTypeFactory<WALL<Coll>, OUTL<Coll>>;
  lb::InitParams ip;
  ip.latDat = &fd.GetDomain();
  ip.lbmParams = &params;
  ip.neighbouringDataManager = nullptr;
  ip.boundaryObject = nullptr;
  Mid s0(ip);
  Wall s1(ip);
  ip.boundaryObject = &inlets;
  Inl s2(ip);
  ip.boundaryObject = &outlets;
  Outl s3(ip);
  ip.boundaryObject = &inlets;
  InlW s4(ip);
  ip.boundaryObject = &outlets;
  OutlW s5(ip);
  lb::MacroscopicPropertyCache cache;
  site_t off[7];
  off[0] = 0;
  for (int t = 0; t < 6; ++t) off[t + 1] = off[t] + counts[t];
  for (int step = 0; step < nsteps; ++step) {
    s0.StreamAndCollide(off[0], counts[0], &params, fd, cache);
    s1.StreamAndCollide(off[1], counts[1], &params, fd, cache);
    s2.StreamAndCollide(off[2], counts[2], &params, fd, cache);
    s3.StreamAndCollide(off[3], counts[3], &params, fd, cache);
    s4.StreamAndCollide(off[4], counts[4], &params, fd, cache);
    s5.StreamAndCollide(off[5], counts[5], &params, fd, cache);
    s0.PostStep(off[0], counts[0], &params, fd, cache);
    s1.PostStep(off[1], counts[1], &params, fd, cache);
    s2.PostStep(off[2], counts[2], &params, fd, cache);
    s3.PostStep(off[3], counts[3], &params, fd, cache);
    s4.PostStep(off[4], counts[4], &params, fd, cache);
    s5.PostStep(off[5], counts[5], &params, fd, cache);
    if (mode == 1 && step == nsteps - 1) break;  // leave fNew un-swapped for inspection
    fd.SwapOldAndNew();
    state.Increment();
  }
  return 0;
}

template <class KERN>
int dispatch(int wall, int inl, int outl, geometry::FieldData& fd, const lb::LbmParameters& p,
             lb::BoundaryValues& bi, lb::BoundaryValues& bo, const site_t c[6],
             lb::SimulationState& st, int n, int mode) {
  using namespace lb;
#define HLB_RUN(W, I, O) return run<KERN, W, I, O>(fd, p, bi, bo, c, st, n, mode)
  if (wall == 0) {
    if (inl == 0 && outl == 0) HLB_RUN(BounceBackLink, NashZerothOrderPressureLink, NashZerothOrderPressureLink);
    if (inl == 1 && outl == 0) HLB_RUN(BounceBackLink, LaddIoletLink, NashZerothOrderPressureLink);
    if (inl == 0 && outl == 1) HLB_RUN(BounceBackLink, NashZerothOrderPressureLink, LaddIoletLink);
    HLB_RUN(BounceBackLink, LaddIoletLink, LaddIoletLink);
  }
  if (inl == 0 && outl == 0)
    HLB_RUN(BouzidiFirdaousLallemandLink, NashZerothOrderPressureLink, NashZerothOrderPressureLink);
  if (inl == 1 && outl == 0)
    HLB_RUN(BouzidiFirdaousLallemandLink, LaddIoletLink, NashZerothOrderPressureLink);
  if (inl == 0 && outl == 1)
    HLB_RUN(BouzidiFirdaousLallemandLink, NashZerothOrderPressureLink, LaddIoletLink);
  HLB_RUN(BouzidiFirdaousLallemandLink, LaddIoletLink, LaddIoletLink);
#undef HLB_RUN
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: %s input.bin output.bin\n", argv[0]);
    return 2;
  }
  FILE* fi = fopen(argv[1], "rb");
  if (!fi) return 3;
  Reader r{fi};
  const int32_t q = r.get<int32_t>();
  const int64_t n = r.get<int64_t>();
  site_t counts[6];
  for (int t = 0; t < 6; ++t) counts[t] = r.get<int64_t>();
  const int32_t kernel = r.get<int32_t>(), wall = r.get<int32_t>(), inl = r.get<int32_t>(),
                outl = r.get<int32_t>();
  const double tau = r.get<double>();
  const int32_t nsteps = r.get<int32_t>();
  const int32_t mode = r.get<int32_t>();
  const uint64_t t_start = r.get<uint64_t>();
  const int32_t n_in = r.get<int32_t>(), n_out = r.get<int32_t>();
  std::vector<IoletIn> ioin((size_t)n_in + n_out);
  for (auto& io : ioin) io = r.get<IoletIn>();
  std::vector<int64_t> nbr, coords;
  std::vector<uint32_t> wm, im;
  std::vector<int32_t> ioid;
  std::vector<int8_t> stype;
  std::vector<double> cut, f0, f1;
  r.arr(nbr, (size_t)n * q);
  r.arr(wm, n);
  r.arr(im, n);
  r.arr(ioid, n);
  r.arr(stype, n);
  r.arr(cut, (size_t)n * (q - 1));
  r.arr(coords, (size_t)n * 3);
  r.arr(f0, (size_t)n * q + 1);
  r.arr(f1, (size_t)n * q + 1);
  fclose(fi);
  if (kernel != 0 && kernel != 1) {
    fprintf(stderr, "kernel must be 0 (LBGK) or 1 (TRT)\n");
    return 4;
  }

  auto dom = std::make_shared<geometry::Domain>();
  dom->n = n;
  dom->siteData.resize(n);
  dom->wallNormalAtSite.assign(n, util::Vector3D<distribn_t>(0.0, 0.0, 0.0));
  dom->globalSiteCoords.resize(n);
  for (int64_t i = 0; i < n; ++i) {
    geometry::SiteData& sd = dom->siteData[i];
    sd.GetWallIntersectionData() = wm[i];
    sd.GetIoletIntersectionData() = im[i];
    sd.GetIoletId() = ioid[i];
    sd.GetSiteType() = (geometry::SiteType)stype[i];
    dom->globalSiteCoords[i] = LatticeVector(coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]);
  }
  dom->distanceToWall = cut;
  dom->neighbourIndices = nbr;
  geometry::FieldData fd;
  fd.m_domain = dom;
  fd.m_currentDistributions = f0;
  fd.m_nextDistributions = f1;
  fd.m_force.assign(n, LatticeForceVector(0.0, 0.0, 0.0));

  // LbmParameters::CalcDerivedParams with unit time step, voxel and density
  lb::LbmParameters params(1.0, 1.0, 1.0, (tau - 0.5) * Cs2);

  lb::SimulationState state;
  state.timeStep = t_start;
  lb::BoundaryValues inlets, outlets;
  inlets.state = &state;
  outlets.state = &state;
  std::vector<std::unique_ptr<lb::InOutLet>> own;
  for (int k = 0; k < n_in + n_out; ++k) {
    own.emplace_back(make_iolet(ioin[k]));
    (k < n_in ? inlets : outlets).iolets.push_back(own.back().get());
  }
  // LBM::PrepareBoundaryObjects (Code/lb/lb.hpp:127-152)
  distribn_t minDensity = std::numeric_limits<distribn_t>::max();
  for (auto* io : inlets.iolets) minDensity = std::min(minDensity, io->GetDensityMin());
  for (auto* io : outlets.iolets) minDensity = std::min(minDensity, io->GetDensityMin());
  for (auto* io : inlets.iolets) io->SetMinimumSimulationDensity(minDensity);
  for (auto* io : outlets.iolets) io->SetMinimumSimulationDensity(minDensity);

  int rc;
#define HLB_DISPATCH(K) dispatch<K>(wall, inl, outl, fd, params, inlets, outlets, counts, state, nsteps, mode)
  if (q == 15)
    rc = kernel == 0 ? HLB_DISPATCH(lb::LBGK<lb::D3Q15>) : HLB_DISPATCH(lb::TRT<lb::D3Q15>);
  else
    rc = kernel == 0 ? HLB_DISPATCH(lb::LBGK<lb::D3Q19>) : HLB_DISPATCH(lb::TRT<lb::D3Q19>);
#undef HLB_DISPATCH
  if (rc) return rc;
  FILE* fo = fopen(argv[2], "wb");
  if (!fo) return 5;
  double tau_used = params.GetTau();
  uint64_t t_end = state.GetTimeStep();
  fwrite(&tau_used, sizeof(double), 1, fo);
  fwrite(&t_end, sizeof(uint64_t), 1, fo);
  fwrite(fd.m_currentDistributions.data(), sizeof(double), fd.m_currentDistributions.size(), fo);
  fwrite(fd.m_nextDistributions.data(), sizeof(double), fd.m_nextDistributions.size(), fo);
  fclose(fo);
  return 0;
}

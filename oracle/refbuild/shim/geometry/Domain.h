// Serial, in-memory stand-in for geometry::Domain holding exactly the arrays the
// LB streamers read (Code/geometry/Domain.h:405-434,487-527): site data, cut
// distances, push table, global coordinates and wall normals.  Filled by the
// driver from the oracle's Domain build.
#ifndef HLB_REFSHIM_GEOMETRY_DOMAIN_H
#define HLB_REFSHIM_GEOMETRY_DOMAIN_H
#include <vector>
#include "units.h"
#include "geometry/SiteData.h"
#include "util/Vector3D.h"
namespace hemelb::geometry {
class Domain {
 public:
  site_t n = 0;
  std::vector<SiteData> siteData;
  std::vector<distribn_t> distanceToWall;
  std::vector<site_t> neighbourIndices;
  std::vector<LatticeVector> globalSiteCoords;
  std::vector<util::Vector3D<distribn_t>> wallNormalAtSite;
  site_t GetLocalFluidSiteCount() const { return n; }
  template <typename LatticeType>
  double GetCutDistance(site_t i, int d) const {
    return distanceToWall[i * (LatticeType::NUMVECTORS - 1) + d - 1];
  }
  const distribn_t* GetCutDistances(site_t i) const { return &distanceToWall[i * 18]; }
  distribn_t* GetCutDistances(site_t i) { return &distanceToWall[i * 18]; }
  template <typename LatticeType>
  site_t GetStreamedIndex(site_t i, unsigned d) const {
    return neighbourIndices[i * LatticeType::NUMVECTORS + d];
  }
  const SiteData& GetSiteData(site_t i) const { return siteData[i]; }
  SiteData& GetSiteData(site_t i) { return siteData[i]; }
  const LatticeVector& GetGlobalSiteCoords(site_t i) const { return globalSiteCoords[i]; }
  const util::Vector3D<distribn_t>& GetNormalToWall(site_t i) const { return wallNormalAtSite[i]; }
  util::Vector3D<distribn_t>& GetNormalToWall(site_t i) { return wallNormalAtSite[i]; }
};
}  // namespace hemelb::geometry
#endif

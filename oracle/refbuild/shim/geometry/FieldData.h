// Serial stand-in for geometry::FieldData (Code/geometry/FieldData.h:27-214):
// fOld / fNew of N*Q+1 doubles and the Site accessors the streamers use.
#ifndef HLB_REFSHIM_GEOMETRY_FIELDDATA_H
#define HLB_REFSHIM_GEOMETRY_FIELDDATA_H
#include <memory>
#include <vector>
#include "units.h"
#include "geometry/Domain.h"
#include "geometry/Site.h"
namespace hemelb::geometry {
class FieldData {
 public:
  using domain_type = Domain;
  std::shared_ptr<Domain> m_domain;
  std::vector<distribn_t> m_currentDistributions, m_nextDistributions;
  std::vector<LatticeForceVector> m_force;
  domain_type const& GetDomain() const { return *m_domain; }
  domain_type& GetDomain() { return *m_domain; }
  Site<FieldData> GetSite(site_t i) { return Site<FieldData>(i, *this); }
  Site<const FieldData> GetSite(site_t i) const { return Site<const FieldData>(i, *this); }
  distribn_t* GetFOld(site_t i) { return &m_currentDistributions[i]; }
  const distribn_t* GetFOld(site_t i) const { return &m_currentDistributions[i]; }
  distribn_t* GetFNew(site_t i) { return &m_nextDistributions[i]; }
  const distribn_t* GetFNew(site_t i) const { return &m_nextDistributions[i]; }
  void SwapOldAndNew() { m_currentDistributions.swap(m_nextDistributions); }
  LatticeForceVector const& GetForceAtSite(site_t i) const { return m_force[i]; }
  void SetForceAtSite(site_t i, LatticeForceVector const& f) { m_force[i] = f; }
  void AddToForceAtSite(site_t i, LatticeForceVector const& f) { m_force[i] += f; }
};
}  // namespace hemelb::geometry
#endif

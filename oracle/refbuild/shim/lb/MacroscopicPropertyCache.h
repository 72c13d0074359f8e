// Property cache with every refresh flag off, as in a run that requests no
// property output (Code/lb/MacroscopicPropertyCache.h:24-90).
#ifndef HLB_REFSHIM_LB_MACROSCOPICPROPERTYCACHE_H
#define HLB_REFSHIM_LB_MACROSCOPICPROPERTYCACHE_H
#include "units.h"
namespace hemelb::lb {
struct NullCache {
  bool RequiresRefresh() const { return false; }
  template <class T> void Put(site_t, T const&) {}
};
class MacroscopicPropertyCache {
 public:
  NullCache densityCache, velocityCache, wallShearStressMagnitudeCache, vonMisesStressCache,
      shearRateCache, stressTensorCache, tractionCache, tangentialProjectionTractionCache;
};
}  // namespace hemelb::lb
#endif

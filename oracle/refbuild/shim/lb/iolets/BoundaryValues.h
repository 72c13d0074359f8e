// Serial BoundaryValues with one rank owning every iolet: the accessors the
// iolet link streamers call (Code/lb/iolets/BoundaryValues.h:43-70,
// BoundaryValues.cc:162-165).
#ifndef HLB_REFSHIM_LB_IOLETS_BOUNDARYVALUES_H
#define HLB_REFSHIM_LB_IOLETS_BOUNDARYVALUES_H
#include <vector>
#include "lb/iolets/InOutLet.h"
#include "lb/SimulationState.h"
namespace hemelb::lb {
class BoundaryValues {
 public:
  std::vector<InOutLet*> iolets;
  const SimulationState* state = nullptr;
  InOutLet* GetLocalIolet(unsigned int i) { return iolets[i]; }
  InOutLet const* GetLocalIolet(unsigned int i) const { return iolets[i]; }
  auto GetLocalIoletCount() const { return iolets.size(); }
  unsigned int GetTimeStep() const { return state->GetTimeStep(); }
  LatticeDensity GetBoundaryDensity(const int index) {
    return iolets[index]->GetDensity(state->Get0IndexedTimeStep());
  }
};
}  // namespace hemelb::lb
#endif

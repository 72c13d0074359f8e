// Serial SimulationState with the reference's time-step semantics
// (Code/lb/SimulationState.cc: starts at 1, Get0IndexedTimeStep = timeStep - 1).
#ifndef HLB_REFSHIM_LB_SIMULATIONSTATE_H
#define HLB_REFSHIM_LB_SIMULATIONSTATE_H
#include "units.h"
namespace hemelb::lb {
enum Stability { UndefinedStability = -1, Unstable = 0, Stable = 1, StableAndConverged = 2 };
class SimulationState {
 public:
  unsigned long timeStep = 1;
  LatticeTimeStep GetTimeStep() const { return timeStep; }
  LatticeTimeStep Get0IndexedTimeStep() const { return timeStep - 1; }
  void Increment() { ++timeStep; }
};
}  // namespace hemelb::lb
#endif

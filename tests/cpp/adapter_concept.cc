// Compile-and-link check: the HemeLB-side plugin types over the C ABI satisfy the
// reference's own concepts when built against its headers.
#include "lb/iolets/BoundaryValues.h"
#include "lb/iolets/InOutLetCosine.h"
#include "lb/iolets/InOutLetParabolicVelocity.h"
#include "lb/lattices/D3Q19.h"
#include "lb/kernels/LBGK.h"
#include "lb/collisions/Normal.h"
#include "lb/streamers/StreamerTypeFactory.h"
#include "hemelb_gb300_hemelb.hpp"

using namespace hemelb;
using Coll = lb::Normal<lb::LBGK<lb::D3Q19>>;
using Gpu = hemelb_gb300::GpuStreamer<Coll>;
static_assert(lb::collision_type<Coll>);
static_assert(lb::streamer<Gpu>, "GpuStreamer must satisfy hemelb::lb::streamer");
static_assert(lb::streamer<lb::BulkStreamer<Coll>>);

int main() {
  // Exercise the reference-independent wrapper without touching a GPU.
  hemelb_gb300::GeometryBuilder gb(19);
  gb.AddFluidSite(3, 3, 3);
  gb.AddFluidSite(3, 3, 4, 0, 1u << 4, 0, HLBG_SITE_INLET);
  const hlbg_geometry& g = gb.View();
  if (g.n_blocks != 1 || g.n_link_sites != 1) return 1;
  return 0;
}

// Runs the LB update through the C++ wrapper (hemelb_gb300.hpp) on a site list
// read from a file, and writes fOld in contiguous site order.
//   wrapper_run <sites.bin> <steps> <out.bin> [<checkpoint.xtr> <more steps> <restart.bin>]
// With a checkpoint path, the state after <steps> is also written as an XTR
// checkpoint, read into a second solver, and both run <more steps>; restart.bin
// then holds [the continued fOld | the restarted fOld | the restarted solver's
// iolet fluxes].
// sites.bin: int64 n, then per site: int64 x,y,z; uint32 wall, iolet; int32 ioid;
// int32 type; float cut[18]; then int32 n_in, n_out and hlbg_iolet records;
// then hlbg_params.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "hemelb_gb300.hpp"

int main(int argc, char** argv) {
  if (argc != 4 && argc != 7) return 2;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 3;
  int64_t n = 0;
  if (fread(&n, 8, 1, f) != 1) return 4;
  hemelb_gb300::GeometryBuilder gb(19);
  for (int64_t i = 0; i < n; ++i) {
    int64_t xyz[3];
    uint32_t wm, im;
    int32_t ioid, type;
    float cut[18];
    if (fread(xyz, 8, 3, f) != 3 || fread(&wm, 4, 1, f) != 1 || fread(&im, 4, 1, f) != 1 ||
        fread(&ioid, 4, 1, f) != 1 || fread(&type, 4, 1, f) != 1 || fread(cut, 4, 18, f) != 18)
      return 5;
    double cd[18];
    for (int k = 0; k < 18; ++k) cd[k] = cut[k];
    gb.AddFluidSite(xyz[0], xyz[1], xyz[2], wm, im, ioid, (int8_t)type, cd);
  }
  int32_t ni = 0, no = 0;
  if (fread(&ni, 4, 1, f) != 1 || fread(&no, 4, 1, f) != 1) return 6;
  std::vector<hlbg_iolet> in(ni), out(no);
  if (ni && fread(in.data(), sizeof(hlbg_iolet), ni, f) != (size_t)ni) return 7;
  if (no && fread(out.data(), sizeof(hlbg_iolet), no, f) != (size_t)no) return 7;
  hlbg_params p{};
  if (fread(&p, sizeof(p), 1, f) != 1) return 8;
  fclose(f);
  try {
    hemelb_gb300::Solver s(gb.View(), p, in, out);
    s.SetEquilibrium();
    s.Step(atoi(argv[2]));
    std::vector<double> fo((size_t)s.SiteCount() * 19);
    s.GetF(fo.data(), 0);
    FILE* o = fopen(argv[3], "wb");
    fwrite(fo.data(), 8, fo.size(), o);
    fclose(o);
    if (argc == 7) {
      const int steps = atoi(argv[2]), more = atoi(argv[5]);
      s.WriteCheckpoint(argv[4], (uint64_t)steps);
      hemelb_gb300::Solver r(gb.View(), p, in, out);
      if (r.ReadCheckpoint(argv[4]) != (uint64_t)steps) return 10;
      r.SetTimeStep((uint64_t)steps + 1);
      s.Step(more);
      r.Step(more);
      std::vector<double> a(fo.size()), b(fo.size());
      s.GetF(a.data(), 0);
      r.GetF(b.data(), 0);
      const std::vector<double> flux = r.IoletFlux();
      FILE* q = fopen(argv[6], "wb");
      fwrite(a.data(), 8, a.size(), q);
      fwrite(b.data(), 8, b.size(), q);
      fwrite(flux.data(), 8, flux.size(), q);
      fclose(q);
    }
  } catch (const hemelb_gb300::Error& e) {
    fprintf(stderr, "%s\n", e.what());
    return 9;
  }
  return 0;
}

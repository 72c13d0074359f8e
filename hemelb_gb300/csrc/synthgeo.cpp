// Seeded synthetic vessel geometries in HemeLB's sparse-block form.
//
// The output is what a GmyReadResult holds after GeometryReader::LoadAndDecompose
// (Code/geometry/GeometryReader.cc:80-166, ParseSite :556-657) for the links the
// LB update reads: per non-empty 8^3 block a fluid bitmap, and for every fluid
// site with a solid neighbour its wall/iolet link masks, iolet id, site type and
// cut distances.  SiteData semantics follow Code/geometry/SiteDataBare.cc:18-68:
// the iolet id is that of the last iolet link in direction order, and the site
// type is INLET if any link is an inlet link, else OUTLET if any is an outlet
// link, else FLUID.
//
// Shapes are unions of cylinders with optional spherical end caps (vessel
// segments and junctions) and z-aligned stenosed pipes with a Gaussian
// narrowing.  A voxel centre (integer coordinates) is fluid when it lies inside
// the union, inside the box, and not beyond any iolet plane.  A link from a
// fluid site to a non-fluid site is an iolet link when its end point lies beyond
// an iolet plane (iolets are tested before walls, as StreamerTypeFactory does),
// otherwise a wall link.  Cut distances are fractions of the link length, the
// convention of geometry-tool's CylinderGenerator
// (geometry-tool/HlbGmyTool/Model/Generation/CylinderGenerator.cpp:265-268):
// exact for iolet planes, and for walls the root of the analytic inside-test
// along the link found by bisection to 1e-12 and stored as float (as .gmy does).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <random>
#include <thread>
#include <vector>

#if HLBG_HAVE_ZLIB
#include <zlib.h>
#endif
#include <cstdio>

#include "../../include/hemelb_gb300.h"

namespace {

constexpr int kBlock = 8;
constexpr int kSitesPerBlock = 512;

const int CX19[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int CY19[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
const int CZ19[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
// D3Q15 (Code/lb/lattices/D3Q15.h): rest, 6 faces, 8 corners.
const int CX15[15] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
const int CY15[15] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, -1, 1, -1, 1};
const int CZ15[15] = {0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, 1, -1, -1, 1};

// Elementary functions of the generators, written with IEEE +, -, *, / and sqrt
// only (this unit is compiled without floating-point contraction), so a seeded
// geometry comes out bit for bit the same on every host: the C library's sin,
// cos, exp and cbrt differ by an ulp between x86_64 and aarch64 builds, and one
// flipped rejection test changes a whole random tree.  Methods: Cody-Waite
// range reduction (W. J. Cody and W. Waite, Software Manual for the Elementary
// Functions, 1980) with the constant split into parts whose products with small
// multiples are exact, then the Taylor series of the reduced argument; the cube
// root by Newton's iteration on a mantissa scaled into [0.5, 4).
namespace det {
template <int N>
struct InvFactorials {
  double c[N + 1];
  constexpr InvFactorials() : c() {
    c[0] = 1.0;
    for (int n = 1; n <= N; ++n) c[n] = c[n - 1] / n;
  }
};
constexpr InvFactorials<24> kInvFact{};

inline double exp(double x) {
  if (x != x) return x;
  if (x > 709.0) return HUGE_VAL;
  if (x < -745.0) return 0.0;
  constexpr double kInvLn2 = 1.44269504088896338700e+00;
  constexpr double kLn2Hi = 6.93147180369123816490e-01;  // ln 2 to 32 bits: k * hi is exact
  constexpr double kLn2Lo = 1.90821492927058770002e-10;  // ln 2 - hi
  const double k = std::floor(x * kInvLn2 + 0.5);
  const double r = (x - k * kLn2Hi) - k * kLn2Lo;  // |r| <= ln 2 / 2 (+ rounding)
  double p = kInvFact.c[16];
  for (int n = 15; n >= 0; --n) p = p * r + kInvFact.c[n];
  return std::ldexp(p, (int)k);
}

// sin and cos of r with |r| <= pi/4 (+ rounding), by their Taylor series
inline double sin_reduced(double r) {
  const double r2 = r * r;
  double p = kInvFact.c[23];
  for (int n = 21; n >= 1; n -= 2) p = p * -r2 + kInvFact.c[n];
  return p * r;
}
inline double cos_reduced(double r) {
  const double r2 = r * r;
  double p = kInvFact.c[24];
  for (int n = 22; n >= 0; n -= 2) p = p * -r2 + kInvFact.c[n];
  return p;
}
// x = k pi/2 + r; pi/2 in three parts, the first two to 33 bits
inline double reduce_half_pi(double x, int* quadrant) {
  constexpr double kInvPio2 = 6.36619772367581382433e-01;
  constexpr double kPio2A = 1.57079632673412561417e+00;
  constexpr double kPio2B = 6.07710050630396597660e-11;
  constexpr double kPio2C = 2.02226624879595063154e-21;
  const double k = std::floor(x * kInvPio2 + 0.5);
  *quadrant = (int)(((long long)k % 4 + 4) % 4);
  return ((x - k * kPio2A) - k * kPio2B) - k * kPio2C;
}
inline double sin(double x) {
  int q;
  const double r = reduce_half_pi(x, &q);
  switch (q) {
    case 0: return sin_reduced(r);
    case 1: return cos_reduced(r);
    case 2: return -sin_reduced(r);
    default: return -cos_reduced(r);
  }
}
inline double cos(double x) {
  int q;
  const double r = reduce_half_pi(x, &q);
  switch (q) {
    case 0: return cos_reduced(r);
    case 1: return -sin_reduced(r);
    case 2: return -cos_reduced(r);
    default: return sin_reduced(r);
  }
}
inline double cbrt(double x) {
  if (x == 0.0 || x != x) return x;
  const double a = x < 0 ? -x : x;
  int e;
  double m = std::frexp(a, &e);  // a = m 2^e, m in [0.5, 1)
  int e3 = e >= 0 ? e / 3 : -((-e + 2) / 3);
  m = std::ldexp(m, e - 3 * e3);  // in [0.5, 4)
  double y = 1.0;
  for (int it = 0; it < 8; ++it) y = y - (y * y * y - m) / (3.0 * y * y);
  const double r = std::ldexp(y, e3);
  return x < 0 ? -r : r;
}
}  // namespace det

struct Vec {
  double x, y, z;
};
inline Vec add(Vec a, Vec b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec sub(Vec a, Vec b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec mul(Vec a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(Vec a, Vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec cross(Vec a, Vec b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline Vec normalised(Vec a) { return mul(a, 1.0 / std::sqrt(dot(a, a))); }

struct Shape {
  int kind;  // 0 = cylinder segment (optional caps), 1 = stenosed z pipe
  Vec a, b;
  double r;
  bool cap_a, cap_b;
  double depth, zc, sigma;  // stenosis
  Vec lo, hi;               // bounding box
};

struct Iolet {
  int outlet;  // 0 inlet, 1 outlet
  int index;   // index in its own list
  Vec pos, n;  // n points into the fluid
  double radius;
  Vec lo, hi;
};

bool inside_shape(const Shape& s, Vec p) {
  if (s.kind == 0) {
    Vec v = sub(s.b, s.a);
    Vec w = sub(p, s.a);
    double l2 = dot(v, v);
    double t = dot(w, v) / l2;
    double r2 = s.r * s.r;
    if (t < 0.0) return s.cap_a && dot(w, w) < r2;
    if (t > 1.0) {
      Vec u = sub(p, s.b);
      return s.cap_b && dot(u, u) < r2;
    }
    Vec perp = sub(w, mul(v, t));
    return dot(perp, perp) < r2;
  }
  // stenosed pipe along z from a.z to b.z, axis through (a.x, a.y)
  if (p.z < s.a.z || p.z > s.b.z) return false;
  double dz = p.z - s.zc;
  double rr = s.r * (1.0 - s.depth * det::exp(-dz * dz / (2.0 * s.sigma * s.sigma)));
  double dx = p.x - s.a.x, dy = p.y - s.a.y;
  return dx * dx + dy * dy < rr * rr;
}

// Signed distance of p inside shape s (positive inside) and the outward unit
// gradient of that distance's complement (the wall normal pointing out of the
// fluid); false where the gradient is undefined (on the axis).
bool shape_normal(const Shape& s, Vec p, double& sd, Vec& n) {
  if (s.kind == 0) {
    const Vec v = sub(s.b, s.a), w = sub(p, s.a);
    double t = dot(w, v) / dot(v, v);
    t = std::min(1.0, std::max(0.0, t));
    const Vec c = sub(w, mul(v, t));
    const double d = std::sqrt(dot(c, c));
    sd = s.r - d;
    if (d < 1e-12) return false;
    n = mul(c, 1.0 / d);
    return true;
  }
  const double dz = p.z - s.zc;
  const double g = det::exp(-dz * dz / (2.0 * s.sigma * s.sigma));
  const double R = s.r * (1.0 - s.depth * g);
  const double dRdz = s.r * s.depth * g * dz / (s.sigma * s.sigma);
  const double dx = p.x - s.a.x, dy = p.y - s.a.y, rho = std::sqrt(dx * dx + dy * dy);
  sd = R - rho;
  if (rho < 1e-12) return false;
  n = normalised(Vec{dx / rho, dy / rho, -dRdz});
  return true;
}

// Signed distance of p from the iolet plane (positive on the fluid side).
inline double iolet_side(const Iolet& io, Vec p) { return dot(sub(p, io.pos), io.n); }

bool beyond_iolet(const Iolet& io, Vec p) {
  double s = iolet_side(io, p);
  if (s >= 0.0 || s < -4.0) return false;
  Vec lat = sub(sub(p, io.pos), mul(io.n, s));
  double lim = io.radius * 1.15 + 1.5;
  return dot(lat, lat) < lim * lim;
}

struct Geometry {
  int q = 19;
  int nb[3] = {0, 0, 0};
  std::vector<Shape> shapes;
  std::vector<Iolet> inlets, outlets;
  // outputs
  std::vector<int32_t> block_coords;
  std::vector<uint64_t> fluid_mask;
  std::vector<int64_t> link_site;
  std::vector<uint32_t> wall_mask, iolet_mask;
  std::vector<int32_t> iolet_id;
  std::vector<int8_t> site_type;
  std::vector<float> cuts;
  std::vector<float> normals;  // per link site: unit wall normal, zero without wall links
  int64_t n_fluid = 0;
  bool with_cuts = false;
  // ensemble: member of each output block and per-member parameters
  std::vector<int32_t> block_member;
  std::vector<double> member_tau;
  std::vector<double> member_shape;  // radius, length, narrowing per member
  std::vector<int64_t> member_sites;
};

uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  // x is the most significant bit of each triple (Code/geometry/LookupTree.h:23-41)
  uint64_t m = 0;
  for (int k = 0; k < 16; ++k) {
    m |= (uint64_t)((x >> k) & 1u) << (3 * k + 2);
    m |= (uint64_t)((y >> k) & 1u) << (3 * k + 1);
    m |= (uint64_t)((z >> k) & 1u) << (3 * k);
  }
  return m;
}

struct BlockOut {
  uint64_t mask[8];
  std::vector<int32_t> local;
  std::vector<uint32_t> wall, iolet;
  std::vector<int32_t> ioid;
  std::vector<int8_t> stype;
  std::vector<float> cuts;
  std::vector<float> normals;
  int64_t nfluid = 0;
};

struct Voxelizer {
  Geometry& g;
  const int* cx;
  const int* cy;
  const int* cz;
  // macro grid of 8x8x8 blocks for candidate culling
  int mg[3];
  std::vector<std::vector<int>> cell_shapes, cell_iolets;  // iolet ids: inlets 0.., outlets offset
  Voxelizer(Geometry& geo) : g(geo) {
    if (g.q == 15) {
      cx = CX15; cy = CY15; cz = CZ15;
    } else {
      cx = CX19; cy = CY19; cz = CZ19;
    }
    for (int a = 0; a < 3; ++a) mg[a] = (g.nb[a] + 7) / 8;
    cell_shapes.resize((size_t)mg[0] * mg[1] * mg[2]);
    cell_iolets.resize(cell_shapes.size());
    auto bin = [&](Vec lo, Vec hi, std::vector<std::vector<int>>& lists, int id) {
      int c0[3], c1[3];
      double l[3] = {lo.x - 2, lo.y - 2, lo.z - 2}, h[3] = {hi.x + 2, hi.y + 2, hi.z + 2};
      for (int a = 0; a < 3; ++a) {
        c0[a] = std::max(0, (int)std::floor(l[a] / 64.0));
        c1[a] = std::min(mg[a] - 1, (int)std::floor(h[a] / 64.0));
      }
      for (int i = c0[0]; i <= c1[0]; ++i)
        for (int j = c0[1]; j <= c1[1]; ++j)
          for (int k = c0[2]; k <= c1[2]; ++k)
            lists[((size_t)i * mg[1] + j) * mg[2] + k].push_back(id);
    };
    for (int s = 0; s < (int)g.shapes.size(); ++s) bin(g.shapes[s].lo, g.shapes[s].hi, cell_shapes, s);
    for (int s = 0; s < (int)g.inlets.size(); ++s) bin(g.inlets[s].lo, g.inlets[s].hi, cell_iolets, s);
    for (int s = 0; s < (int)g.outlets.size(); ++s)
      bin(g.outlets[s].lo, g.outlets[s].hi, cell_iolets, (int)g.inlets.size() + s);
  }
  const Iolet& iolet_by(int id) const {
    return id < (int)g.inlets.size() ? g.inlets[id] : g.outlets[id - g.inlets.size()];
  }
  bool in_box(Vec p) const {
    return p.x >= -0.5 && p.y >= -0.5 && p.z >= -0.5 && p.x <= g.nb[0] * kBlock - 0.5 &&
           p.y <= g.nb[1] * kBlock - 0.5 && p.z <= g.nb[2] * kBlock - 0.5;
  }
  bool in_union(const std::vector<int>& shp, Vec p) const {
    for (int s : shp)
      if (inside_shape(g.shapes[s], p)) return true;
    return false;
  }
  bool fluid(const std::vector<int>& shp, const std::vector<int>& iol, Vec p) const {
    if (!in_box(p)) return false;
    if (!in_union(shp, p)) return false;
    for (int i : iol)
      if (beyond_iolet(iolet_by(i), p)) return false;
    return true;
  }

  void block(int bx, int by, int bz, BlockOut& out) const {
    std::memset(out.mask, 0, sizeof(out.mask));
    size_t cell = ((size_t)(bx / 8) * mg[1] + by / 8) * mg[2] + bz / 8;
    const auto& shp = cell_shapes[cell];
    const auto& iol = cell_iolets[cell];
    if (shp.empty()) return;
    // quick reject: block AABB vs candidate shapes' boxes
    double o[3] = {(double)bx * kBlock, (double)by * kBlock, (double)bz * kBlock};
    bool any = false;
    for (int s : shp) {
      const Shape& S = g.shapes[s];
      if (S.hi.x < o[0] - 1.5 || S.lo.x > o[0] + 8.5 || S.hi.y < o[1] - 1.5 ||
          S.lo.y > o[1] + 8.5 || S.hi.z < o[2] - 1.5 || S.lo.z > o[2] + 8.5)
        continue;
      any = true;
      break;
    }
    if (!any) return;
    // fluid flags on a 10^3 halo grid
    uint8_t fl[10][10][10];
    for (int i = 0; i < 10; ++i)
      for (int j = 0; j < 10; ++j)
        for (int k = 0; k < 10; ++k)
          fl[i][j][k] = fluid(shp, iol, Vec{o[0] + i - 1, o[1] + j - 1, o[2] + k - 1});
    const int nl = g.q - 1;
    for (int i = 0; i < 8; ++i)
      for (int j = 0; j < 8; ++j)
        for (int k = 0; k < 8; ++k) {
          if (!fl[i + 1][j + 1][k + 1]) continue;
          int l = (i * 8 + j) * 8 + k;
          out.mask[l >> 6] |= 1ull << (l & 63);
          out.nfluid++;
          uint32_t wm = 0, im = 0;
          int ioid = -1;
          bool had_in = false, had_out = false;
          float cutv[26];
          int hitv[26];
          for (int d = 1; d <= nl; ++d) cutv[d - 1] = -1.0f;  // NO_VALUE-like for fluid links
          for (int d = 1; d <= nl; ++d) hitv[d - 1] = -1;
          Vec p{o[0] + i, o[1] + j, o[2] + k};
          for (int d = 1; d <= nl; ++d) {
            if (fl[i + 1 + cx[d]][j + 1 + cy[d]][k + 1 + cz[d]]) continue;
            Vec c{(double)cx[d], (double)cy[d], (double)cz[d]};
            Vec pe = add(p, c);
            int hit = -1;
            for (int ii : iol)
              if (beyond_iolet(iolet_by(ii), pe)) {
                hit = ii;
                break;
              }
            hitv[d - 1] = hit;
            if (hit >= 0) {
              const Iolet& io = iolet_by(hit);
              im |= 1u << (d - 1);
              ioid = io.index;
              if (io.outlet) had_out = true; else had_in = true;
              double s0 = iolet_side(io, p), s1 = iolet_side(io, pe);
              cutv[d - 1] = (float)(s0 / (s0 - s1));
            } else {
              wm |= 1u << (d - 1);
              if (g.with_cuts) {
                double t0 = 0.0, t1 = 1.0;
                for (int it = 0; it < 48 && t1 - t0 > 1e-12; ++it) {
                  double tm = 0.5 * (t0 + t1);
                  Vec pm = add(p, mul(c, tm));
                  if (in_box(pm) && in_union(shp, pm)) t0 = tm; else t1 = tm;
                }
                double qv = 0.5 * (t0 + t1);
                if (qv < 1e-6) qv = 1e-6;
                cutv[d - 1] = (float)qv;
              }
            }
          }
          if (had_in && had_out) {
            // A site with links to an inlet and to an outlet (an outlet plane that
            // ends next to an inlet): SiteData holds one iolet id for a site typed
            // INLET, so its outlet links become wall links (cut at the link's end).
            ioid = -1;
            for (int d = 1; d <= nl; ++d) {
              if (!((im >> (d - 1)) & 1u)) continue;
              const Iolet& io = iolet_by(hitv[d - 1]);
              if (io.outlet) {
                im &= ~(1u << (d - 1));
                wm |= 1u << (d - 1);
                cutv[d - 1] = 1.0f;
              } else {
                ioid = io.index;
              }
            }
            had_out = false;
          }
          if (wm == 0 && im == 0) continue;
          // wall normal: gradient of the shape the site lies deepest in; else the
          // normalised sum of the wall-link vectors
          Vec nrm{0, 0, 0};
          if (wm) {
            double best = -1e30;
            bool got = false;
            for (int sh : shp) {
              double sdv;
              Vec nv;
              if (shape_normal(g.shapes[sh], p, sdv, nv) && sdv > best) {
                best = sdv;
                nrm = nv;
                got = true;
              }
            }
            if (!got) {
              Vec acc{0, 0, 0};
              for (int d = 1; d <= nl; ++d)
                if ((wm >> (d - 1)) & 1u) acc = add(acc, Vec{(double)cx[d], (double)cy[d], (double)cz[d]});
              if (dot(acc, acc) > 0) nrm = normalised(acc);
            }
          }
          out.normals.push_back((float)nrm.x);
          out.normals.push_back((float)nrm.y);
          out.normals.push_back((float)nrm.z);
          out.local.push_back(l);
          out.wall.push_back(wm);
          out.iolet.push_back(im);
          out.ioid.push_back(ioid);
          out.stype.push_back(had_in ? HLBG_SITE_INLET : (had_out ? HLBG_SITE_OUTLET : HLBG_SITE_FLUID));
          if (g.with_cuts)
            for (int d = 0; d < nl; ++d) out.cuts.push_back(cutv[d]);
        }
  }
};

void shape_bounds(Shape& s) {
  if (s.kind == 0) {
    double r = s.r + 1.0;
    s.lo = {std::min(s.a.x, s.b.x) - r, std::min(s.a.y, s.b.y) - r, std::min(s.a.z, s.b.z) - r};
    s.hi = {std::max(s.a.x, s.b.x) + r, std::max(s.a.y, s.b.y) + r, std::max(s.a.z, s.b.z) + r};
  } else {
    double r = s.r + 1.0;
    s.lo = {s.a.x - r, s.a.y - r, s.a.z - 1.0};
    s.hi = {s.a.x + r, s.a.y + r, s.b.z + 1.0};
  }
}
void iolet_bounds(Iolet& io) {
  double r = io.radius * 1.15 + 6.0;
  io.lo = {io.pos.x - r, io.pos.y - r, io.pos.z - r};
  io.hi = {io.pos.x + r, io.pos.y + r, io.pos.z + r};
}

// Translate everything by an integer offset so the bounding box starts at 2 and
// choose the block counts.
void place(Geometry& g, int fixed_box_sites) {
  if (fixed_box_sites > 0) {
    for (int a = 0; a < 3; ++a) g.nb[a] = fixed_box_sites / kBlock;
  } else {
    Vec lo{1e30, 1e30, 1e30}, hi{-1e30, -1e30, -1e30};
    for (auto& s : g.shapes) {
      shape_bounds(s);
      lo = {std::min(lo.x, s.lo.x), std::min(lo.y, s.lo.y), std::min(lo.z, s.lo.z)};
      hi = {std::max(hi.x, s.hi.x), std::max(hi.y, s.hi.y), std::max(hi.z, s.hi.z)};
    }
    Vec off{2.0 - std::floor(lo.x), 2.0 - std::floor(lo.y), 2.0 - std::floor(lo.z)};
    for (auto& s : g.shapes) {
      s.a = add(s.a, off);
      s.b = add(s.b, off);
      if (s.kind == 1) s.zc += off.z;
    }
    for (auto* v : {&g.inlets, &g.outlets})
      for (auto& io : *v) io.pos = add(io.pos, off);
    double ext[3] = {hi.x + off.x + 3.0, hi.y + off.y + 3.0, hi.z + off.z + 3.0};
    for (int a = 0; a < 3; ++a) g.nb[a] = (int)std::ceil(ext[a] / kBlock);
  }
  for (auto& s : g.shapes) shape_bounds(s);
  for (auto* v : {&g.inlets, &g.outlets})
    for (auto& io : *v) iolet_bounds(io);
}

int voxelize(Geometry& g, int n_threads) {
  Voxelizer vx(g);
  // candidate blocks: those touched by a shape's box
  std::vector<uint8_t> cand((size_t)g.nb[0] * g.nb[1] * g.nb[2], 0);
  for (auto& s : g.shapes) {
    int b0[3], b1[3];
    double l[3] = {s.lo.x - 1, s.lo.y - 1, s.lo.z - 1}, h[3] = {s.hi.x + 1, s.hi.y + 1, s.hi.z + 1};
    for (int a = 0; a < 3; ++a) {
      b0[a] = std::max(0, (int)std::floor(l[a] / kBlock));
      b1[a] = std::min(g.nb[a] - 1, (int)std::floor(h[a] / kBlock));
    }
    for (int i = b0[0]; i <= b1[0]; ++i)
      for (int j = b0[1]; j <= b1[1]; ++j)
        for (int k = b0[2]; k <= b1[2]; ++k) cand[((size_t)i * g.nb[1] + j) * g.nb[2] + k] = 1;
  }
  std::vector<std::pair<uint64_t, uint32_t>> order;  // (morton, block id)
  for (int i = 0; i < g.nb[0]; ++i)
    for (int j = 0; j < g.nb[1]; ++j)
      for (int k = 0; k < g.nb[2]; ++k) {
        size_t id = ((size_t)i * g.nb[1] + j) * g.nb[2] + k;
        if (cand[id]) order.push_back({morton3(i, j, k), (uint32_t)id});
      }
  std::sort(order.begin(), order.end());
  std::vector<BlockOut> outs(order.size());
  std::atomic<size_t> next{0};
  if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
  auto work = [&]() {
    for (;;) {
      size_t c = next.fetch_add(64);
      if (c >= order.size()) break;
      size_t e = std::min(order.size(), c + 64);
      for (size_t t = c; t < e; ++t) {
        uint32_t id = order[t].second;
        int k = id % g.nb[2];
        int j = (id / g.nb[2]) % g.nb[1];
        int i = id / ((size_t)g.nb[2] * g.nb[1]);
        vx.block(i, j, k, outs[t]);
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < n_threads; ++t) th.emplace_back(work);
  work();
  for (auto& t : th) t.join();
  for (size_t t = 0; t < order.size(); ++t) {
    BlockOut& b = outs[t];
    if (b.nfluid == 0) continue;
    uint32_t id = order[t].second;
    int64_t bi = (int64_t)g.block_coords.size() / 3;
    g.block_coords.push_back(id / (g.nb[2] * g.nb[1]));
    g.block_coords.push_back((id / g.nb[2]) % g.nb[1]);
    g.block_coords.push_back(id % g.nb[2]);
    for (int w = 0; w < 8; ++w) g.fluid_mask.push_back(b.mask[w]);
    g.n_fluid += b.nfluid;
    for (size_t s = 0; s < b.local.size(); ++s) {
      g.link_site.push_back(bi * kSitesPerBlock + b.local[s]);
      g.wall_mask.push_back(b.wall[s]);
      g.iolet_mask.push_back(b.iolet[s]);
      g.iolet_id.push_back(b.ioid[s]);
      g.site_type.push_back(b.stype[s]);
    }
    if (g.with_cuts) g.cuts.insert(g.cuts.end(), b.cuts.begin(), b.cuts.end());
    g.normals.insert(g.normals.end(), b.normals.begin(), b.normals.end());
    outs[t] = BlockOut();
  }
  return HLBG_OK;
}

Shape cyl(Vec a, Vec b, double r, bool ca, bool cb) {
  Shape s{};
  s.kind = 0;
  s.a = a;
  s.b = b;
  s.r = r;
  s.cap_a = ca;
  s.cap_b = cb;
  return s;
}
Iolet mk_iolet(int outlet, int index, Vec pos, Vec n, double r) {
  Iolet io{};
  io.outlet = outlet;
  io.index = index;
  io.pos = pos;
  io.n = normalised(n);
  io.radius = r;
  return io;
}

// Unit vector at angle theta from dir, azimuth phi around it.
Vec deflect(Vec dir, double theta, double phi) {
  Vec helper = std::fabs(dir.x) < 0.9 ? Vec{1, 0, 0} : Vec{0, 1, 0};
  Vec e1 = normalised(cross(dir, helper));
  Vec e2 = cross(dir, e1);
  Vec lat = add(mul(e1, det::cos(phi)), mul(e2, det::sin(phi)));
  return normalised(add(mul(dir, det::cos(theta)), mul(lat, det::sin(theta))));
}

int finish(Geometry* g, int n_threads, void** handle) {
  int rc = voxelize(*g, n_threads);
  if (rc != HLBG_OK) {
    delete g;
    return rc;
  }
  *handle = g;
  return HLBG_OK;
}

}  // namespace

extern "C" {

int hlbg_synth_pipe(double radius, int32_t length, int32_t q, int32_t with_cuts, void** handle) {
  if (!handle || radius <= 0 || length < 1 || (q != 15 && q != 19)) return HLBG_ERR_INVAL;
  auto* g = new Geometry();
  g->q = q;
  g->with_cuts = with_cuts != 0;
  g->shapes.push_back(cyl({0, 0, -0.5}, {0, 0, length + 0.5}, radius, false, false));
  g->inlets.push_back(mk_iolet(0, 0, {0, 0, -0.5}, {0, 0, 1}, radius));
  g->outlets.push_back(mk_iolet(1, 0, {0, 0, length + 0.5}, {0, 0, -1}, radius));
  place(*g, 0);
  return finish(g, 0, handle);
}

int hlbg_synth_stenosis(double radius, int32_t length, double depth, int32_t q, int32_t with_cuts,
                        void** handle) {
  if (!handle || radius <= 0 || length < 4 || depth < 0 || depth >= 1 || (q != 15 && q != 19))
    return HLBG_ERR_INVAL;
  auto* g = new Geometry();
  g->q = q;
  g->with_cuts = with_cuts != 0;
  Shape s{};
  s.kind = 1;
  s.a = {0, 0, -0.5};
  s.b = {0, 0, length + 0.5};
  s.r = radius;
  s.depth = depth;
  s.zc = 0.5 * length;
  s.sigma = std::max(2.0, radius);
  g->shapes.push_back(s);
  g->inlets.push_back(mk_iolet(0, 0, {0, 0, -0.5}, {0, 0, 1}, radius));
  g->outlets.push_back(mk_iolet(1, 0, {0, 0, length + 0.5}, {0, 0, -1}, radius));
  place(*g, 0);
  return finish(g, 0, handle);
}

int hlbg_synth_bifurcation(uint64_t seed, double parent_radius, double parent_length,
                           double daughter_length_factor, int32_t q, int32_t with_cuts,
                           void** handle) {
  if (!handle || parent_radius <= 0 || parent_length <= 0 || (q != 15 && q != 19))
    return HLBG_ERR_INVAL;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  double split = 0.3 + 0.4 * U(rng);
  double half = (25.0 + 35.0 * U(rng)) * M_PI / 180.0;
  double r1 = parent_radius * det::cbrt(split), r2 = parent_radius * det::cbrt(1.0 - split);
  auto* g = new Geometry();
  g->q = q;
  g->with_cuts = with_cuts != 0;
  Vec a{0, 0, -0.5}, b{0, 0, parent_length};
  g->shapes.push_back(cyl(a, b, parent_radius, false, true));
  g->inlets.push_back(mk_iolet(0, 0, a, {0, 0, 1}, parent_radius));
  double ld = daughter_length_factor * parent_length;
  Vec d1{det::sin(half), 0, det::cos(half)}, d2{-det::sin(half), 0, det::cos(half)};
  Vec e1 = add(b, mul(d1, ld)), e2 = add(b, mul(d2, ld));
  g->shapes.push_back(cyl(b, e1, r1, true, false));
  g->shapes.push_back(cyl(b, e2, r2, true, false));
  g->outlets.push_back(mk_iolet(1, 0, e1, mul(d1, -1.0), r1));
  g->outlets.push_back(mk_iolet(1, 1, e2, mul(d2, -1.0), r2));
  place(*g, 0);
  return finish(g, 0, handle);
}

int hlbg_synth_tree(uint64_t seed, int32_t box_sites, int32_t n_roots, int32_t depth,
                    double root_radius, int32_t q, int32_t with_cuts, int32_t n_threads,
                    void** handle) {
  if (!handle || box_sites < 64 || box_sites % kBlock || n_roots < 1 || depth < 0 || depth > 12 ||
      root_radius <= 1 || (q != 15 && q != 19))
    return HLBG_ERR_INVAL;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  auto* g = new Geometry();
  g->q = q;
  g->with_cuts = with_cuts != 0;
  const double B = box_sites;
  const double margin = 4.0;
  auto clip_len = [&](Vec p, Vec d, double len) {
    // largest t <= len keeping p + t d inside [margin, B-1-margin]^3
    double t = len;
    double pc[3] = {p.x, p.y, p.z}, dc[3] = {d.x, d.y, d.z};
    for (int a = 0; a < 3; ++a) {
      if (dc[a] > 1e-12) t = std::min(t, (B - 1 - margin - pc[a]) / dc[a]);
      if (dc[a] < -1e-12) t = std::min(t, (margin - pc[a]) / dc[a]);
    }
    return std::max(0.0, t);
  };
  struct Seg {
    Vec start, dir;
    double r;
    int level;
  };
  int n_out = 0;
  for (int root = 0; root < n_roots; ++root) {
    // roots enter through the z=0 face on a jittered grid, pointing inwards
    int gside = (int)std::ceil(std::sqrt((double)n_roots));
    int gi = root % gside, gj = root / gside;
    double cxr = B * (gi + 0.5) / gside + (U(rng) - 0.5) * B * 0.1 / gside;
    double cyr = B * (gj + 0.5) / gside + (U(rng) - 0.5) * B * 0.1 / gside;
    double rr = root_radius;
    cxr = std::min(std::max(cxr, rr + margin + 2), B - rr - margin - 3);
    cyr = std::min(std::max(cyr, rr + margin + 2), B - rr - margin - 3);
    Vec start{cxr, cyr, margin};
    // two draws in sequence: the order in which a call's arguments are evaluated is
    // unspecified (it differs between the x86_64 and aarch64 compilers)
    const double tilt = 10.0 * M_PI / 180.0 * U(rng);
    const double azimuth = 2 * M_PI * U(rng);
    Vec dir = deflect({0, 0, 1}, tilt, azimuth);
    g->inlets.push_back(mk_iolet(0, root, start, dir, rr));
    std::vector<Seg> stack{{start, dir, rr, 0}};
    while (!stack.empty()) {
      Seg s = stack.back();
      stack.pop_back();
      double len = (6.0 + 4.0 * U(rng)) * s.r;
      double l = clip_len(s.start, s.dir, len);
      bool leaf = s.level >= depth || l < 2.0 * s.r;
      if (l < 1.0) l = 1.0;
      Vec end = add(s.start, mul(s.dir, l));
      g->shapes.push_back(cyl(s.start, end, s.r, s.level > 0, !leaf));
      if (leaf) {
        g->outlets.push_back(mk_iolet(1, n_out++, end, mul(s.dir, -1.0), s.r));
        continue;
      }
      double split = 0.3 + 0.4 * U(rng);
      double r1 = s.r * det::cbrt(split), r2 = s.r * det::cbrt(1.0 - split);
      double phi = 2 * M_PI * U(rng);
      double th1 = (20.0 + 50.0 * U(rng)) * M_PI / 180.0;
      double th2 = (20.0 + 50.0 * U(rng)) * M_PI / 180.0;
      Vec d1 = deflect(s.dir, th1, phi), d2 = deflect(s.dir, th2, phi + M_PI);
      // steer children that would leave the box straight away back towards the centre
      Vec centre{B / 2, B / 2, B / 2};
      for (Vec* d : {&d1, &d2}) {
        if (clip_len(end, *d, 6.0 * s.r) < 3.0 * s.r) {
          Vec to_c = normalised(sub(centre, end));
          *d = normalised(add(*d, mul(to_c, 1.5)));
        }
      }
      stack.push_back({end, d2, r2, s.level + 1});
      stack.push_back({end, d1, r1, s.level + 1});
    }
  }
  place(*g, box_sites);
  return finish(g, n_threads, handle);
}

int hlbg_synth_ensemble(uint64_t seed, int32_t n_members, int32_t q, int32_t n_threads,
                        void** handle) {
  // Seeded stenosed pipes: radius U[6,20], length U[60,240], Gaussian narrowing
  // U[0,0.7] of the radius, tau U[0.55,1.0].  Each member occupies its own cell of
  // blocks in a 2-D arrangement over (x, y), cells separated by one empty block so
  // that no link joins two members.  Inlet i / outlet i belong to member i.
  if (!handle || n_members < 1 || n_members > 65536 || (q != 15 && q != 19)) return HLBG_ERR_INVAL;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  auto* g = new Geometry();
  g->q = q;
  g->with_cuts = true;
  const int cell_xy = 6;   // blocks: 2 * 20 + margins fits in 5 blocks, plus a 1-block gap
  const int cell_z = 32;   // blocks: length <= 240 + margins fits in 31, plus a gap
  const int side = (int)std::ceil(std::sqrt((double)n_members));
  std::vector<std::unique_ptr<Geometry>> members;
  for (int m = 0; m < n_members; ++m) {
    double R = 6.0 + 14.0 * U(rng);
    int L = 60 + (int)std::floor(181.0 * U(rng));
    double depth = 0.7 * U(rng);
    double tau = 0.55 + 0.45 * U(rng);
    auto mg = std::make_unique<Geometry>();
    mg->q = q;
    mg->with_cuts = true;
    Shape sh{};
    sh.kind = 1;
    sh.a = {0, 0, -0.5};
    sh.b = {0, 0, L + 0.5};
    sh.r = R;
    sh.depth = depth;
    sh.zc = 0.5 * L;
    sh.sigma = std::max(2.0, R);
    mg->shapes.push_back(sh);
    mg->inlets.push_back(mk_iolet(0, m, {0, 0, -0.5}, {0, 0, 1}, R));
    mg->outlets.push_back(mk_iolet(1, m, {0, 0, L + 0.5}, {0, 0, -1}, R));
    // centre the pipe in its cell: axis at 8*cell_xy/2 - 4 sites from the cell corner
    Vec off{(double)(cell_xy * 8 / 2 - 4), (double)(cell_xy * 8 / 2 - 4), 3.0};
    for (auto& sp : mg->shapes) {
      sp.a = add(sp.a, off);
      sp.b = add(sp.b, off);
      sp.zc += off.z;
    }
    for (auto* v : {&mg->inlets, &mg->outlets})
      for (auto& io : *v) io.pos = add(io.pos, off);
    mg->nb[0] = mg->nb[1] = cell_xy - 1;
    mg->nb[2] = cell_z - 1;
    for (auto& sp : mg->shapes) shape_bounds(sp);
    for (auto* v : {&mg->inlets, &mg->outlets})
      for (auto& io : *v) iolet_bounds(io);
    g->member_tau.push_back(tau);
    g->member_shape.push_back(R);
    g->member_shape.push_back((double)L);
    g->member_shape.push_back(depth);
    members.push_back(std::move(mg));
  }
  // voxelise members in parallel
  std::atomic<int> next{0};
  if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
  auto work = [&]() {
    for (;;) {
      int m = next.fetch_add(1);
      if (m >= n_members) break;
      voxelize(*members[m], 1);
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < n_threads; ++t) th.emplace_back(work);
  work();
  for (auto& t : th) t.join();
  g->nb[0] = side * cell_xy;
  g->nb[1] = side * cell_xy;
  g->nb[2] = cell_z;
  const int nl = q - 1;
  for (int m = 0; m < n_members; ++m) {
    Geometry& mg = *members[m];
    const int ox = (m % side) * cell_xy, oy = (m / side) * cell_xy;
    const int64_t b0 = (int64_t)g->block_coords.size() / 3;
    const int64_t nbm = (int64_t)mg.block_coords.size() / 3;
    for (int64_t b = 0; b < nbm; ++b) {
      g->block_coords.push_back(mg.block_coords[3 * b] + ox);
      g->block_coords.push_back(mg.block_coords[3 * b + 1] + oy);
      g->block_coords.push_back(mg.block_coords[3 * b + 2]);
      g->block_member.push_back(m);
    }
    g->fluid_mask.insert(g->fluid_mask.end(), mg.fluid_mask.begin(), mg.fluid_mask.end());
    for (size_t r = 0; r < mg.link_site.size(); ++r) {
      g->link_site.push_back(mg.link_site[r] + b0 * kSitesPerBlock);
      g->wall_mask.push_back(mg.wall_mask[r]);
      g->iolet_mask.push_back(mg.iolet_mask[r]);
      g->iolet_id.push_back(mg.iolet_id[r] >= 0 ? m : -1);
      g->site_type.push_back(mg.site_type[r]);
    }
    g->cuts.insert(g->cuts.end(), mg.cuts.begin(), mg.cuts.end());
    g->normals.insert(g->normals.end(), mg.normals.begin(), mg.normals.end());
    g->n_fluid += mg.n_fluid;
    g->member_sites.push_back(mg.n_fluid);
    Vec shift{8.0 * ox, 8.0 * oy, 0.0};
    for (auto io : mg.inlets) {
      io.pos = add(io.pos, shift);
      io.index = m;
      g->inlets.push_back(io);
    }
    for (auto io : mg.outlets) {
      io.pos = add(io.pos, shift);
      io.index = m;
      g->outlets.push_back(io);
    }
  }
  (void)nl;
  *handle = g;
  return HLBG_OK;
}

int hlbg_synth_members(void* handle, int32_t* n_members, const int32_t** block_member,
                       const double** member_tau, const double** member_shape,
                       const int64_t** member_sites) {
  if (!handle) return HLBG_ERR_INVAL;
  auto* g = static_cast<Geometry*>(handle);
  if (n_members) *n_members = (int32_t)g->member_tau.size();
  if (block_member) *block_member = g->block_member.empty() ? nullptr : g->block_member.data();
  if (member_tau) *member_tau = g->member_tau.empty() ? nullptr : g->member_tau.data();
  if (member_shape) *member_shape = g->member_shape.empty() ? nullptr : g->member_shape.data();
  if (member_sites) *member_sites = g->member_sites.empty() ? nullptr : g->member_sites.data();
  return HLBG_OK;
}

// ---------------------------------------------------------------------------
// HemeLB .gmy geometry files (doc/dev/file-formats/geometry.md; the reader of the
// reference is Code/geometry/GeometryReader.cc:80-166 and ParseSite :556-657).
// XDR big-endian words: preamble (magics 0x686c6221 / 0x676d7904, version 4,
// block counts, block size, pad), one (fluid sites, compressed bytes,
// uncompressed bytes) header per block with z fastest, then the zlib-compressed
// site records of every non-empty block, sites with z fastest.  A fluid site
// carries 26 links over the Moore neighbourhood in lexicographic (x, y, z)
// order without the rest vector: cut type (0 none, 1 wall, 2 inlet, 3 outlet),
// then an iolet index for inlets/outlets and a float cut distance for all but
// none; then a wall-normal flag and, if set, the normal.
// ---------------------------------------------------------------------------
namespace {
struct XdrIn {
  const uint8_t* p;
  size_t n, at = 0;
  bool ok = true;
  uint32_t u32() {
    if (at + 4 > n) {
      ok = false;
      return 0;
    }
    uint32_t v = ((uint32_t)p[at] << 24) | ((uint32_t)p[at + 1] << 16) | ((uint32_t)p[at + 2] << 8) |
                 (uint32_t)p[at + 3];
    at += 4;
    return v;
  }
  float f32() {
    uint32_t v = u32();
    float f;
    std::memcpy(&f, &v, 4);
    return f;
  }
};
}  // namespace

extern "C" {
int hlbg_read_gmy(const char* path, int32_t q, void** handle) {
  if (!path || !handle || (q != 15 && q != 19)) return HLBG_ERR_INVAL;
#if !HLBG_HAVE_ZLIB
  (void)path;
  return HLBG_ERR_STATE;  // built without zlib
#else
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return HLBG_ERR_INVAL;
  std::vector<uint8_t> file;
  {
    uint8_t buf[1 << 16];
    size_t r;
    while ((r = std::fread(buf, 1, sizeof(buf), fp)) > 0) file.insert(file.end(), buf, buf + r);
    std::fclose(fp);
  }
  XdrIn in{file.data(), file.size()};
  const uint32_t m1 = in.u32(), m2 = in.u32(), ver = in.u32();
  const uint32_t nbx = in.u32(), nby = in.u32(), nbz = in.u32(), bs = in.u32();
  in.u32();
  if (!in.ok || m1 != 0x686c6221u || m2 != 0x676d7904u || ver != 4 || bs == 0 || bs > 64)
    return HLBG_ERR_INVAL;
  const uint64_t nblk = (uint64_t)nbx * nby * nbz;
  std::vector<uint32_t> hdr(nblk * 3);
  for (auto& h : hdr) h = in.u32();
  if (!in.ok) return HLBG_ERR_INVAL;
  // lattice direction of each of the 26 Moore links (0 = not in the lattice)
  const int* cx = q == 15 ? CX15 : CX19;
  const int* cy = q == 15 ? CY15 : CY19;
  const int* cz = q == 15 ? CZ15 : CZ19;
  int link_dir[26];
  {
    int i = 0;
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          if (!dx && !dy && !dz) continue;
          link_dir[i] = 0;
          for (int d = 1; d < q; ++d)
            if (cx[d] == dx && cy[d] == dy && cz[d] == dz) link_dir[i] = d;
          ++i;
        }
  }
  struct SiteRec {
    int64_t x, y, z;
    uint32_t wall, iolet;
    int32_t ioid;
    int8_t type;
    float cut[26];
    float normal[3];
  };
  std::vector<SiteRec> sites;
  size_t off = in.at;
  std::vector<uint8_t> raw;
  for (uint64_t b = 0; b < nblk; ++b) {
    const uint32_t nsite = hdr[3 * b], clen = hdr[3 * b + 1], ulen = hdr[3 * b + 2];
    if (nsite == 0) continue;
    if (off + clen > file.size()) return HLBG_ERR_INVAL;
    raw.assign(ulen, 0);
    uLongf got = ulen;
    if (uncompress(raw.data(), &got, file.data() + off, clen) != Z_OK || got != ulen) return HLBG_ERR_INVAL;
    off += clen;
    const int64_t bx = (int64_t)(b / ((uint64_t)nby * nbz)), by = (int64_t)((b / nbz) % nby),
                  bz = (int64_t)(b % nbz);
    XdrIn s{raw.data(), raw.size()};
    uint32_t seen = 0;
    for (uint32_t lx = 0; lx < bs; ++lx)
      for (uint32_t ly = 0; ly < bs; ++ly)
        for (uint32_t lz = 0; lz < bs; ++lz) {
          const uint32_t fluid = s.u32();
          if (!s.ok || fluid > 1) return HLBG_ERR_INVAL;
          if (!fluid) continue;
          SiteRec r{};
          r.x = bx * bs + lx;
          r.y = by * bs + ly;
          r.z = bz * bs + lz;
          r.ioid = -1;
          bool had_in = false, had_out = false, any_wall = false;
          for (int d = 0; d < 26; ++d) r.cut[d] = -1.0f;  // GeometrySiteLink default
          for (int i = 0; i < 26; ++i) {
            const uint32_t type = s.u32();
            int32_t io = -1;
            float dist = -1.0f;
            if (type == 1) {
              dist = s.f32();
              any_wall = true;
            } else if (type == 2 || type == 3) {
              io = (int32_t)s.u32();
              dist = s.f32();
            } else if (type != 0) {
              return HLBG_ERR_INVAL;
            }
            const int d = link_dir[i];
            if (d == 0) continue;  // link not in this lattice
            r.cut[d - 1] = dist;
            if (type == 1) r.wall |= 1u << (d - 1);
            if (type == 2 || type == 3) {
              r.iolet |= 1u << (d - 1);
              r.ioid = io;  // SiteData: the last iolet link in direction order wins
              if (type == 2) had_in = true; else had_out = true;
            }
          }
          const uint32_t has_normal = s.u32();
          if (has_normal > 1 || (has_normal == 1) != any_wall) return HLBG_ERR_INVAL;
          r.normal[0] = r.normal[1] = r.normal[2] = 0.f;
          if (has_normal) {
            r.normal[0] = s.f32();
            r.normal[1] = s.f32();
            r.normal[2] = s.f32();
          }
          if (!s.ok) return HLBG_ERR_INVAL;
          r.type = had_in ? HLBG_SITE_INLET : (had_out ? HLBG_SITE_OUTLET : HLBG_SITE_FLUID);
          sites.push_back(r);
          ++seen;
        }
    if (seen != nsite) return HLBG_ERR_INVAL;
  }
  // re-block into 8^3 blocks, listed in Morton order
  auto* g = new Geometry();
  g->q = q;
  g->with_cuts = true;
  int64_t ext[3] = {(int64_t)nbx * bs, (int64_t)nby * bs, (int64_t)nbz * bs};
  for (int a = 0; a < 3; ++a) g->nb[a] = (int)((ext[a] + kBlock - 1) / kBlock);
  std::vector<std::pair<uint64_t, size_t>> order;
  order.reserve(sites.size());
  for (size_t i = 0; i < sites.size(); ++i) {
    const auto& r = sites[i];
    uint64_t key = (morton3((uint32_t)(r.x >> 3), (uint32_t)(r.y >> 3), (uint32_t)(r.z >> 3)) << 9) |
                   (uint64_t)(((r.x & 7) * 8 + (r.y & 7)) * 8 + (r.z & 7));
    order.push_back({key, i});
  }
  std::sort(order.begin(), order.end());
  uint64_t cur_block = ~0ull;
  int64_t bi = -1;
  for (auto& [key, i] : order) {
    const auto& r = sites[i];
    const uint64_t blk = key >> 9;
    if (blk != cur_block) {
      cur_block = blk;
      ++bi;
      g->block_coords.push_back((int32_t)(r.x >> 3));
      g->block_coords.push_back((int32_t)(r.y >> 3));
      g->block_coords.push_back((int32_t)(r.z >> 3));
      for (int w = 0; w < 8; ++w) g->fluid_mask.push_back(0);
    }
    const int l = (int)(key & 511);
    g->fluid_mask[bi * 8 + l / 64] |= 1ull << (l % 64);
    g->n_fluid++;
    if (r.wall || r.iolet) {
      g->link_site.push_back(bi * kSitesPerBlock + l);
      g->wall_mask.push_back(r.wall);
      g->iolet_mask.push_back(r.iolet);
      g->iolet_id.push_back(r.ioid);
      g->site_type.push_back(r.type);
      for (int d = 0; d < q - 1; ++d) g->cuts.push_back(r.cut[d]);
      for (int c = 0; c < 3; ++c) g->normals.push_back(r.normal[c]);
    }
  }
  *handle = g;
  return HLBG_OK;
#endif
}
}  // extern "C"

int hlbg_write_gmy(const hlbg_geometry* g, const char* path) {
  // Inverse of hlbg_read_gmy with 8^3 blocks.  Lattice links keep their cut type,
  // iolet index and distance; Moore links outside the lattice are written as
  // NONE.  Sites with a wall link get a wall normal (the geometry's own, else the
  // normalised sum of their wall-link vectors), as the format requires one exactly
  // for wall sites.
#if !HLBG_HAVE_ZLIB
  (void)g;
  (void)path;
  return HLBG_ERR_STATE;
#else
  if (!g || !path || (g->q != 15 && g->q != 19) || g->block_size != 8) return HLBG_ERR_INVAL;
  const int q = g->q;
  const int* cx = q == 15 ? CX15 : CX19;
  const int* cy = q == 15 ? CY15 : CY19;
  const int* cz = q == 15 ? CZ15 : CZ19;
  int dir_of_link[26];
  {
    int i = 0;
    for (int dx = -1; dx <= 1; ++dx)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dz = -1; dz <= 1; ++dz) {
          if (!dx && !dy && !dz) continue;
          dir_of_link[i] = 0;
          for (int d = 1; d < q; ++d)
            if (cx[d] == dx && cy[d] == dy && cz[d] == dz) dir_of_link[i] = d;
          ++i;
        }
  }
  const uint64_t NX = g->blocks[0], NY = g->blocks[1], NZ = g->blocks[2];
  std::vector<int64_t> idx(NX * NY * NZ, -1);
  for (int64_t b = 0; b < g->n_blocks; ++b)
    idx[((uint64_t)g->block_coords[3 * b] * NY + g->block_coords[3 * b + 1]) * NZ + g->block_coords[3 * b + 2]] = b;
  std::vector<int64_t> rec_of(g->n_blocks * 512, -1);
  for (int64_t r = 0; r < g->n_link_sites; ++r) rec_of[g->link_site[r]] = r;
  auto put = [](std::vector<uint8_t>& v, uint32_t w) {
    v.push_back((uint8_t)(w >> 24));
    v.push_back((uint8_t)(w >> 16));
    v.push_back((uint8_t)(w >> 8));
    v.push_back((uint8_t)w);
  };
  auto putf = [&](std::vector<uint8_t>& v, float f) {
    uint32_t w;
    std::memcpy(&w, &f, 4);
    put(v, w);
  };
  std::vector<uint8_t> head, body;
  put(head, 0x686c6221u);
  put(head, 0x676d7904u);
  put(head, 4u);
  put(head, (uint32_t)NX);
  put(head, (uint32_t)NY);
  put(head, (uint32_t)NZ);
  put(head, 8u);
  put(head, 0u);
  std::vector<uint8_t> raw;
  for (uint64_t gb = 0; gb < NX * NY * NZ; ++gb) {
    const int64_t b = idx[gb];
    if (b < 0) {
      put(head, 0u);
      put(head, 0u);
      put(head, 0u);
      continue;
    }
    raw.clear();
    uint32_t nfluid = 0;
    for (int l = 0; l < 512; ++l) {
      const bool fl = (g->fluid_mask[b * 8 + l / 64] >> (l % 64)) & 1ull;
      put(raw, fl ? 1u : 0u);
      if (!fl) continue;
      ++nfluid;
      const int64_t r = rec_of[b * 512 + l];
      double nx = 0, ny = 0, nz = 0;
      bool any_wall = false;
      for (int i = 0; i < 26; ++i) {
        const int d = dir_of_link[i];
        uint32_t type = 0;
        if (d && r >= 0) {
          const bool w = (g->wall_mask[r] >> (d - 1)) & 1u, io = (g->iolet_mask[r] >> (d - 1)) & 1u;
          const float dist = g->cut_distance ? g->cut_distance[r * (q - 1) + d - 1] : 0.5f;
          if (io) {
            type = g->site_type[r] == HLBG_SITE_OUTLET ? 3u : 2u;
            put(raw, type);
            put(raw, (uint32_t)std::max(0, g->iolet_id[r]));
            putf(raw, dist);
            continue;
          }
          if (w) {
            put(raw, 1u);
            putf(raw, dist);
            any_wall = true;
            nx += cx[d];
            ny += cy[d];
            nz += cz[d];
            continue;
          }
        }
        put(raw, 0u);
      }
      put(raw, any_wall ? 1u : 0u);
      if (any_wall && g->wall_normal) {  // the geometry's own normal, as it is
        for (int c = 0; c < 3; ++c) putf(raw, g->wall_normal[3 * r + c]);
      } else if (any_wall) {
        double m = std::sqrt(nx * nx + ny * ny + nz * nz);
        if (m == 0) m = 1;
        putf(raw, (float)(nx / m));
        putf(raw, (float)(ny / m));
        putf(raw, (float)(nz / m));
      }
    }
    uLongf clen = compressBound(raw.size());
    std::vector<uint8_t> comp(clen);
    if (compress(comp.data(), &clen, raw.data(), raw.size()) != Z_OK) return HLBG_ERR_INVAL;
    put(head, nfluid);
    put(head, (uint32_t)clen);
    put(head, (uint32_t)raw.size());
    body.insert(body.end(), comp.begin(), comp.begin() + clen);
  }
  FILE* fp = std::fopen(path, "wb");
  if (!fp) return HLBG_ERR_INVAL;
  bool ok = std::fwrite(head.data(), 1, head.size(), fp) == head.size() &&
            std::fwrite(body.data(), 1, body.size(), fp) == body.size();
  ok = (std::fclose(fp) == 0) && ok;
  return ok ? HLBG_OK : HLBG_ERR_INVAL;
#endif
}

int hlbg_synth_view(void* handle, hlbg_geometry* out, int64_t* n_fluid, int32_t* n_in,
                    int32_t* n_outl) {
  if (!handle || !out) return HLBG_ERR_INVAL;
  auto* g = static_cast<Geometry*>(handle);
  std::memset(out, 0, sizeof(*out));
  out->q = g->q;
  out->block_size = kBlock;
  for (int a = 0; a < 3; ++a) out->blocks[a] = g->nb[a];
  out->n_blocks = (int64_t)g->block_coords.size() / 3;
  out->block_coords = g->block_coords.data();
  out->fluid_mask = g->fluid_mask.data();
  out->n_link_sites = (int64_t)g->link_site.size();
  out->link_site = g->link_site.data();
  out->wall_mask = g->wall_mask.data();
  out->iolet_mask = g->iolet_mask.data();
  out->iolet_id = g->iolet_id.data();
  out->site_type = g->site_type.data();
  out->cut_distance = g->with_cuts ? g->cuts.data() : nullptr;
  out->wall_normal = g->normals.size() == 3 * g->link_site.size() && !g->normals.empty() ? g->normals.data() : nullptr;
  if (n_fluid) *n_fluid = g->n_fluid;
  if (n_in) *n_in = (int32_t)g->inlets.size();
  if (n_outl) *n_outl = (int32_t)g->outlets.size();
  return HLBG_OK;
}

int hlbg_synth_iolet(void* handle, int32_t is_outlet, int32_t index, double position[3],
                     double normal[3], double* radius) {
  if (!handle) return HLBG_ERR_INVAL;
  auto* g = static_cast<Geometry*>(handle);
  const auto& v = is_outlet ? g->outlets : g->inlets;
  if (index < 0 || index >= (int)v.size()) return HLBG_ERR_INVAL;
  const Iolet& io = v[index];
  position[0] = io.pos.x;
  position[1] = io.pos.y;
  position[2] = io.pos.z;
  normal[0] = io.n.x;
  normal[1] = io.n.y;
  normal[2] = io.n.z;
  if (radius) *radius = io.radius;
  return HLBG_OK;
}

void hlbg_synth_free(void* handle) { delete static_cast<Geometry*>(handle); }

// One seeded vessel in a fixed cubic box of box_sites^3 voxels (a multiple of 8);
// lengths below are for a 96 box and scale with box_sites / 96:
// kind 0 a stenosed pipe along z (radius U[6,14], Gaussian narrowing of depth
// U[0,0.6] and width U[0.5,1.5] x radius, centre z in U[0.35,0.65] x box, axis
// offset up to 10 sites from the box centre); kind 1 a bifurcation (parent radius
// U[6,12] along z up to a split at U[0.3,0.5] x box, Murray daughters with split
// ratio U[0.3,0.7], half-angles U[20,45] degrees in a random plane, each running
// to the box margin).  Inlet plane z = 1.5 (normal +z), outlets at the far ends.
// Simple bounce-back geometry (no cut distances).
int hlbg_synth_vessel_box(uint64_t seed, int32_t box_sites, int32_t kind, int32_t q, void** handle) {
  if (!handle || box_sites < 32 || box_sites % kBlock || (kind != 0 && kind != 1) || (q != 15 && q != 19))
    return HLBG_ERR_INVAL;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  const double B = box_sites;
  const double sc = B / 96.0;
  auto* g = new Geometry();
  g->q = q;
  g->with_cuts = false;
  const double z_in = 1.5;
  const Vec axis0{0.5 * B - 0.5 + (U(rng) - 0.5) * 20.0 * sc, 0.5 * B - 0.5 + (U(rng) - 0.5) * 20.0 * sc, 0.0};
  if (kind == 0) {
    const double r = (6.0 + 8.0 * U(rng)) * sc;
    Shape s{};
    s.kind = 1;
    s.a = {axis0.x, axis0.y, z_in - 1.0};
    s.b = {axis0.x, axis0.y, B - 1.5};
    s.r = r;
    s.depth = 0.6 * U(rng);
    s.zc = (0.35 + 0.3 * U(rng)) * B;
    s.sigma = (0.5 + U(rng)) * r;
    g->shapes.push_back(s);
    g->inlets.push_back(mk_iolet(0, 0, {axis0.x, axis0.y, z_in}, {0, 0, 1}, r));
    g->outlets.push_back(mk_iolet(1, 0, {axis0.x, axis0.y, B - 2.5}, {0, 0, -1}, r));
  } else {
    const double r0 = (6.0 + 6.0 * U(rng)) * sc;
    const double zs = (0.3 + 0.2 * U(rng)) * B;
    const double split = 0.3 + 0.4 * U(rng);
    const double th1 = (20.0 + 25.0 * U(rng)) * M_PI / 180.0, th2 = (20.0 + 25.0 * U(rng)) * M_PI / 180.0;
    const double phi = 2.0 * M_PI * U(rng);
    const double r1 = r0 * det::cbrt(split), r2 = r0 * det::cbrt(1.0 - split);
    const Vec a{axis0.x, axis0.y, z_in - 1.0}, b{axis0.x, axis0.y, zs};
    g->shapes.push_back(cyl(a, b, r0, false, true));
    g->inlets.push_back(mk_iolet(0, 0, {axis0.x, axis0.y, z_in}, {0, 0, 1}, r0));
    const Vec zdir{0, 0, 1};
    const Vec dirs[2] = {deflect(zdir, th1, phi), deflect(zdir, th2, phi + M_PI)};
    const double rs[2] = {r1, r2};
    for (int k = 0; k < 2; ++k) {
      // run to the margin: lateral faces r + 3 sites in, top face 2.5 sites in
      const Vec d = dirs[k];
      const double m = rs[k] + 3.0 * sc;
      double len = 1e30;
      const double lo[3] = {m, m, 0.0}, hi[3] = {B - 1.0 - m, B - 1.0 - m, B - 2.5};
      const double p0[3] = {b.x, b.y, b.z}, dv[3] = {d.x, d.y, d.z};
      for (int ax = 0; ax < 3; ++ax) {
        if (dv[ax] > 1e-9) len = std::min(len, (hi[ax] - p0[ax]) / dv[ax]);
        if (dv[ax] < -1e-9) len = std::min(len, (lo[ax] - p0[ax]) / dv[ax]);
      }
      len = std::max(len, 2.0 * rs[k]);
      const Vec e = add(b, mul(d, len));
      g->shapes.push_back(cyl(b, e, rs[k], true, false));
      g->outlets.push_back(mk_iolet(1, k, e, mul(d, -1.0), rs[k]));
    }
  }
  place(*g, box_sites);
  return finish(g, 0, handle);
}

// Signed distance to the vessel wall at every voxel centre of the box (positive
// inside): for each shape its radius (local radius for the stenosed pipe) minus
// the distance to its axis segment, the largest over shapes.  out holds
// box^3 floats, x slowest and z fastest.
int hlbg_synth_distance(void* handle, float* out) {
  if (!handle || !out) return HLBG_ERR_INVAL;
  auto* g = static_cast<Geometry*>(handle);
  const int X = g->nb[0] * kBlock, Y = g->nb[1] * kBlock, Z = g->nb[2] * kBlock;
  for (int x = 0; x < X; ++x)
    for (int y = 0; y < Y; ++y)
      for (int z = 0; z < Z; ++z) {
        const Vec p{(double)x, (double)y, (double)z};
        double best = -1e30;
        for (const Shape& s : g->shapes) {
          double sd;
          if (s.kind == 0) {
            const Vec v = sub(s.b, s.a), w = sub(p, s.a);
            double t = dot(w, v) / dot(v, v);
            t = std::min(1.0, std::max(0.0, t));
            const Vec c = sub(w, mul(v, t));
            sd = s.r - std::sqrt(dot(c, c));
          } else {
            const double dz = p.z - s.zc;
            const double rr = s.r * (1.0 - s.depth * det::exp(-dz * dz / (2.0 * s.sigma * s.sigma)));
            const double dx = p.x - s.a.x, dy = p.y - s.a.y;
            sd = rr - std::sqrt(dx * dx + dy * dy);
          }
          best = std::max(best, sd);
        }
        out[((size_t)x * Y + y) * Z + z] = (float)best;
      }
  return HLBG_OK;
}

}  // extern "C"

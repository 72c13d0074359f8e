/*
 * CPU oracle for the HemeLB lattice-Boltzmann update -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, in plain C and in the reference's floating-point evaluation order,
 * the per-step sweep of lb::LBM (Code/lb/lb.hpp:176-309) with the pieces it
 * calls.  Each function cites the reference file:line it follows.  Compiled with
 * -ffp-contract=off so that no multiply-add is fused: every + and * rounds
 * separately, exactly as written in the reference sources.
 *
 * Used only by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
 */
#include "hlb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* Code/constants.h:18,41 */
static const double kPI = 3.14159265358979323846264338327950288;
static const double kCs2 = 1.0 / 3.0;

/* Code/lb/lattices/D3Q19.h:14-49 */
static const int CX19[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int CY19[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int CZ19[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
static const double W19[19] = {1.0 / 3.0,  1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 18.0,
                               1.0 / 18.0, 1.0 / 18.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                               1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0,
                               1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
/* Code/lb/lattices/D3Q15.h:14-50 */
static const int CX15[15] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
static const int CY15[15] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, -1, 1, -1, 1};
static const int CZ15[15] = {0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, 1, -1, -1, 1};
static const double W15[15] = {2.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,  1.0 / 9.0,
                               1.0 / 9.0,  1.0 / 9.0,  1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0,
                               1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0, 1.0 / 72.0};

typedef struct {
  int q;
  const int *cx, *cy, *cz;
  const double *w;
  int inv[19];
} lat_t;

static void lattice(int q, lat_t *L) {
  L->q = q;
  if (q == 15) {
    L->cx = CX15; L->cy = CY15; L->cz = CZ15; L->w = W15;
  } else {
    L->cx = CX19; L->cy = CY19; L->cz = CZ19; L->w = W19;
  }
  /* Code/lb/lattices/Lattice.h:49-69 compute_inverses */
  for (int i = 0; i < q; ++i)
    for (int j = i; j < q; ++j)
      if (L->cx[i] == -L->cx[j] && L->cy[i] == -L->cy[j] && L->cz[i] == -L->cz[j]) {
        L->inv[i] = j;
        L->inv[j] = i;
      }
}

/* ---- Lattice math -------------------------------------------------------- */

/* Code/lb/lattices/Lattice.h:181-191 (scalar) and :119-178 (SSE3 lane order:
 * the low lane sums the even directions from 0, the high lane starts from the
 * odd last direction and then sums the odd directions; a horizontal add joins
 * them as low + high). */
static void density_momentum(const lat_t *L, int order, const double *f, double *rho,
                             double m[3]) {
  const int q = L->q;
  if (order == HLBO_ORDER_SCALAR) {
    double r = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
    for (int i = 0; i < q; ++i) {
      r += f[i];
      /* momentum += VECTORS[i] * f[i]: Vector3D<int> * double -> {cx*f, cy*f, cz*f} */
      mx += (double)L->cx[i] * f[i];
      my += (double)L->cy[i] * f[i];
      mz += (double)L->cz[i] * f[i];
    }
    *rho = r;
    m[0] = mx; m[1] = my; m[2] = mz;
    return;
  }
  int n2 = (q >> 1) << 1;
  double rl = 0.0, rh = 0.0, xl = 0.0, xh = 0.0, yl = 0.0, yh = 0.0, zl = 0.0, zh = 0.0;
  if (q != n2) {
    rh = f[q - 1];
    xh = (double)L->cx[q - 1] * f[q - 1];
    yh = (double)L->cy[q - 1] * f[q - 1];
    zh = (double)L->cz[q - 1] * f[q - 1];
  }
  for (int i = 0; i < n2; i += 2) {
    rl = rl + f[i];
    rh = rh + f[i + 1];
    xl = xl + (double)L->cx[i] * f[i];
    xh = xh + (double)L->cx[i + 1] * f[i + 1];
    yl = yl + (double)L->cy[i] * f[i];
    yh = yh + (double)L->cy[i + 1] * f[i + 1];
    zl = zl + (double)L->cz[i] * f[i];
    zh = zh + (double)L->cz[i + 1] * f[i + 1];
  }
  *rho = rl + rh;
  m[0] = xl + xh;
  m[1] = yl + yh;
  m[2] = zl + zh;
}

/* Code/lb/lattices/Lattice.h:332-355 (scalar, compressible) and :236-321 (SSE3). */
static void feq_of(const lat_t *L, int order, double rho, const double m[3], double *feq) {
  const int q = L->q;
  const double mx = m[0], my = m[1], mz = m[2];
  if (order == HLBO_ORDER_SCALAR) {
    const double density_1 = 1. / rho;
    const double m2 = mx * mx + my * my + mz * mz;
    for (int i = 0; i < q; ++i) {
      const double mde = L->cx[i] * mx + L->cy[i] * my + L->cz[i] * mz;
      feq[i] = L->w[i] * (rho - (3. / 2.) * m2 * density_1 + (9. / 2.) * density_1 * mde * mde +
                          3. * mde);
    }
    return;
  }
  const double threeHalves = (3. / 2.) * (mx * mx + my * my + mz * mz);
  const double tmp1 = rho - threeHalves / rho;
  const double density_1 = 1. / rho;
  double nineHalves = (9. / 2.);
  nineHalves *= density_1;
  for (int i = 0; i < q; ++i) {
    /* both the paired lanes and the odd last direction use this association */
    const double mde = ((double)L->cx[i] * mx + (double)L->cy[i] * my) + (double)L->cz[i] * mz;
    const double t2 = nineHalves * (mde * mde);
    const double t3 = 3. * mde;
    feq[i] = L->w[i] * ((tmp1 + t2) + t3);
  }
}

void hlbo_feq(const hlbo_params *p, double density, const double mom[3], double *feq) {
  lat_t L;
  lattice(p->q, &L);
  feq_of(&L, p->order, density, mom, feq);
}

/* HydroVars + Kernel: LBGK (Code/lb/kernels/LBGK.h:29-63) or TRT
 * (Code/lb/kernels/TRT.h:94-122, magic parameter 3/16).  TRT's moments are
 * LBGK's (Lattice.h:471-483, the overload TRT.h:62-92 means to call), f_neq =
 * f - f_eq, the rest direction relaxed with omega+ (TRT.h:108-112) and the nine
 * opposite pairs (i, iBar) with i < iBar relaxed with omega+/omega- in the
 * order of TRT.h:115-121.  Pinned bit for bit to the reference's TRT.h compiled
 * with the build-time patch of oracle/refbuild/build_ref.py. */
static void collide(const lat_t *L, const hlbo_params *p, const double *f, double *rho,
                    double m[3], double u[3], double *feq, double *fpost) {
  const int q = L->q;
  double fneq[19];
  density_momentum(L, p->order, f, rho, m);
  u[0] = m[0] / *rho;
  u[1] = m[1] / *rho;
  u[2] = m[2] / *rho;
  feq_of(L, p->order, *rho, m, feq);
  for (int i = 0; i < q; ++i) fneq[i] = f[i] - feq[i];
  const double omega = -1.0 / p->tau; /* Code/lb/LbmParameters.h:36 */
  if (p->kernel == HLBG_KERNEL_LBGK) {
    for (int i = 0; i < q; ++i) fpost[i] = f[i] + fneq[i] * omega;
    return;
  }
  const double Lambda = 3.0 / 16.0;
  const double tau_plus = p->tau;
  const double omega_plus = omega;
  const double tau_minus = 0.5 + Lambda / (tau_plus - 0.5);
  const double omega_minus = -1.0 / tau_minus;
  fpost[0] = f[0] + omega_plus * fneq[0];
  for (int i = 1; i < q; ++i) {
    int ib = L->inv[i];
    if (ib < i) continue;
    double sym = 0.5 * omega_plus * (fneq[i] + fneq[ib]);
    double asym = 0.5 * omega_minus * (fneq[i] - fneq[ib]);
    fpost[i] = f[i] + sym + asym;
    fpost[ib] = f[ib] + sym - asym;
  }
}

void hlbo_collide_site(const hlbo_params *p, const double *f, double *density, double *mom,
                       double *vel, double *feq, double *fpost) {
  lat_t L;
  lattice(p->q, &L);
  collide(&L, p, f, density, mom, vel, feq, fpost);
}

/* ---- iolet values ---------------------------------------------------------- */

static double dot3(const double a[3], const double b[3]) {
  /* std::inner_product from RES{0} (Code/util/Vector3D.h:381-386) */
  double s = 0.0;
  s = s + a[0] * b[0];
  s = s + a[1] * b[1];
  s = s + a[2] * b[2];
  return s;
}

static double density_min_of(const hlbg_iolet *io) {
  /* InOutLetCosine::GetDensityMin (InOutLetCosine.h:50-53); velocity iolets 1.0
   * (InOutLetVelocity.cc:17-20) */
  if (io->model == HLBG_IOLET_COSINE) return io->density_mean - io->density_amp;
  return 1.0;
}

double hlbo_min_density(const hlbo_params *p) {
  /* LBM::PrepareBoundaryObjects (Code/lb/lb.hpp:127-152) */
  double m = 1.7976931348623157e308;
  for (int i = 0; i < p->n_inlets; ++i) {
    double v = density_min_of(&p->inlets[i]);
    m = v < m ? v : m;
  }
  for (int i = 0; i < p->n_outlets; ++i) {
    double v = density_min_of(&p->outlets[i]);
    m = v < m ? v : m;
  }
  return m;
}

double hlbo_cosine_density(const hlbg_iolet *io, uint64_t t, double min_density) {
  /* InOutLetCosine::GetDensity (Code/lb/iolets/InOutLetCosine.cc:26-43) */
  if (io->model != HLBG_IOLET_COSINE) return 1.0; /* InOutLetVelocity::GetDensity */
  double w = 2.0 * kPI / io->period;
  double target = io->density_mean + io->density_amp * cos(w * (double)t + io->phase);
  if (t >= io->warmup_steps) return target;
  double interp = ((double)t) / ((double)io->warmup_steps);
  return interp * target + (1. - interp) * min_density;
}

static void normalise(const double in[3], double out[3]) {
  /* Vector3D::GetNormalised: divide by sqrt(Dot(v, v)) (Code/util/Vector3D.h:300-339) */
  double mag = sqrt(dot3(in, in));
  out[0] = in[0] / mag;
  out[1] = in[1] / mag;
  out[2] = in[2] / mag;
}

void hlbo_iolet_velocity(const hlbg_iolet *io, const double x[3], uint64_t t, double out[3]) {
  /* InOutLetParabolicVelocity::GetVelocity (Code/lb/iolets/InOutLetParabolicVelocity.cc:23-43).
   * The pulsatile model scales the peak by (1 - cos(2 pi t / T)) / 2 before the
   * same warm-up and profile. */
  double n[3];
  normalise(io->normal, n);
  double displ[3] = {x[0] - io->position[0], x[1] - io->position[1], x[2] - io->position[2]};
  double z = dot3(displ, n);
  double rSq = (dot3(displ, displ) - z * z) / (io->radius * io->radius);
  double max = io->max_speed;
  if (io->model == HLBG_IOLET_PULSATILE)
    max = max * (0.5 * (1.0 - cos(2.0 * kPI * (double)t / io->vel_period)));
  if (t < io->warmup_steps) max *= (double)t / (double)io->warmup_steps;
  double s = max * (1. - rSq);
  out[0] = n[0] * s;
  out[1] = n[1] * s;
  out[2] = n[2] * s;
}

/* ---- domain construction ------------------------------------------------- */

static uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  /* Code/geometry/LookupTree.h:23-41: x is the most significant bit of each triple */
  uint64_t m = 0;
  for (int k = 0; k < 16; ++k) {
    m |= (uint64_t)((x >> k) & 1u) << (3 * k + 2);
    m |= (uint64_t)((y >> k) & 1u) << (3 * k + 1);
    m |= (uint64_t)((z >> k) & 1u) << (3 * k);
  }
  return m;
}

typedef struct {
  uint64_t key;
  int64_t idx;
} kv_t;
static int kv_cmp(const void *a, const void *b) {
  const kv_t *x = (const kv_t *)a, *y = (const kv_t *)b;
  return x->key < y->key ? -1 : (x->key > y->key ? 1 : 0);
}

static int collision_type_of(uint32_t wall, int8_t type) {
  /* SiteData::GetCollisionType (Code/geometry/SiteDataBare.cc:102-145) and the
   * index mapping of Domain::ProcessReadSites (Code/geometry/Domain.cc:188-207) */
  if (wall == 0) return type == HLBG_SITE_INLET ? 2 : (type == HLBG_SITE_OUTLET ? 3 : 0);
  return type == HLBG_SITE_INLET ? 4 : (type == HLBG_SITE_OUTLET ? 5 : 1);
}

int hlbo_domain_build(const hlbg_geometry *g, hlbo_domain *d) {
  memset(d, 0, sizeof(*d));
  const int q = g->q;
  if ((q != 15 && q != 19) || g->block_size != 8) return HLBG_ERR_INVAL;
  lat_t L;
  lattice(q, &L);
  const int64_t nb = g->n_blocks;
  /* blocks in octree leaf (Morton) order */
  kv_t *bo = (kv_t *)malloc(sizeof(kv_t) * (nb ? nb : 1));
  for (int64_t b = 0; b < nb; ++b) {
    bo[b].key = morton3(g->block_coords[3 * b], g->block_coords[3 * b + 1],
                        g->block_coords[3 * b + 2]);
    bo[b].idx = b;
  }
  qsort(bo, nb, sizeof(kv_t), kv_cmp);
  /* per slot: link record index (or -1) */
  int64_t nslot = nb * 512;
  int64_t *rec = (int64_t *)malloc(sizeof(int64_t) * (nslot ? nslot : 1));
  for (int64_t s = 0; s < nslot; ++s) rec[s] = -1;
  for (int64_t r = 0; r < g->n_link_sites; ++r) rec[g->link_site[r]] = r;
  /* count fluid sites by type */
  int64_t n = 0;
  int64_t cnt[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t s = 0; s < nslot; ++s) {
    int64_t b = s >> 9, l = s & 511;
    if (!((g->fluid_mask[b * 8 + (l >> 6)] >> (l & 63)) & 1ull)) continue;
    int64_t r = rec[s];
    int t = r < 0 ? 0 : collision_type_of(g->wall_mask[r], g->site_type[r]);
    cnt[t]++;
    n++;
  }
  d->q = q;
  d->n = n;
  for (int t = 0; t < 6; ++t) d->type_count[t] = cnt[t];
  d->nbr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n * q > 0 ? n * q : 1));
  d->wall_mask = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
  d->iolet_mask = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
  d->iolet_id = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
  d->site_type = (int8_t *)malloc(n ? n : 1);
  d->cut = (double *)malloc(sizeof(double) * (size_t)(n * (q - 1) > 0 ? n * (q - 1) : 1));
  d->coords = (int64_t *)malloc(sizeof(int64_t) * 3 * (n ? n : 1));
  d->slot = (int64_t *)malloc(sizeof(int64_t) * (n ? n : 1));
  /* contiguous ids: type by type; inside a type in block (Morton) then site order
   * (Domain::PopulateWithReadData, Code/geometry/Domain.cc:288-357) */
  int64_t off[6];
  off[0] = 0;
  for (int t = 1; t < 6; ++t) off[t] = off[t - 1] + cnt[t - 1];
  int64_t *id_of_slot = (int64_t *)malloc(sizeof(int64_t) * (nslot ? nslot : 1));
  for (int64_t s = 0; s < nslot; ++s) id_of_slot[s] = -1;
  for (int64_t bi = 0; bi < nb; ++bi) {
    int64_t b = bo[bi].idx;
    for (int l = 0; l < 512; ++l) {
      if (!((g->fluid_mask[b * 8 + (l >> 6)] >> (l & 63)) & 1ull)) continue;
      int64_t s = b * 512 + l;
      int64_t r = rec[s];
      int t = r < 0 ? 0 : collision_type_of(g->wall_mask[r], g->site_type[r]);
      int64_t id = off[t]++;
      id_of_slot[s] = id;
      d->slot[id] = s;
      d->coords[3 * id + 0] = (int64_t)g->block_coords[3 * b + 0] * 8 + (l >> 6);
      d->coords[3 * id + 1] = (int64_t)g->block_coords[3 * b + 1] * 8 + ((l >> 3) & 7);
      d->coords[3 * id + 2] = (int64_t)g->block_coords[3 * b + 2] * 8 + (l & 7);
      if (r >= 0) {
        d->wall_mask[id] = g->wall_mask[r];
        d->iolet_mask[id] = g->iolet_mask[r];
        d->iolet_id[id] = g->iolet_id[r];
        d->site_type[id] = g->site_type[r];
        for (int k = 0; k < q - 1; ++k)
          d->cut[id * (q - 1) + k] = g->cut_distance ? (double)g->cut_distance[r * (q - 1) + k]
                                                     : -1.0;
      } else {
        d->wall_mask[id] = 0;
        d->iolet_mask[id] = 0;
        d->iolet_id[id] = -1;
        d->site_type[id] = HLBG_SITE_FLUID;
        for (int k = 0; k < q - 1; ++k) d->cut[id * (q - 1) + k] = -1.0;
      }
    }
  }
  /* block lookup by coordinates for the neighbour table */
  const int64_t NX = g->blocks[0], NY = g->blocks[1], NZ = g->blocks[2];
  int64_t *blk = (int64_t *)malloc(sizeof(int64_t) * (size_t)(NX * NY * NZ));
  for (int64_t i = 0; i < NX * NY * NZ; ++i) blk[i] = -1;
  for (int64_t b = 0; b < nb; ++b)
    blk[((int64_t)g->block_coords[3 * b] * NY + g->block_coords[3 * b + 1]) * NZ +
        g->block_coords[3 * b + 2]] = b;
  /* Domain::InitialiseNeighbourLookup (Code/geometry/Domain.cc:425-505) */
  for (int64_t id = 0; id < n; ++id) {
    d->nbr[id * q + 0] = id * q + 0;
    for (int dd = 1; dd < q; ++dd) {
      int64_t x = d->coords[3 * id] + L.cx[dd], y = d->coords[3 * id + 1] + L.cy[dd],
              z = d->coords[3 * id + 2] + L.cz[dd];
      int64_t target = n * q; /* rubbish site */
      if (x >= 0 && y >= 0 && z >= 0 && x < NX * 8 && y < NY * 8 && z < NZ * 8) {
        int64_t b = blk[((x >> 3) * NY + (y >> 3)) * NZ + (z >> 3)];
        if (b >= 0) {
          int64_t s = b * 512 + (((x & 7) * 8 + (y & 7)) * 8 + (z & 7));
          if (id_of_slot[s] >= 0) target = id_of_slot[s] * q + dd;
        }
      }
      d->nbr[id * q + dd] = target;
    }
  }
  free(blk);
  free(id_of_slot);
  free(rec);
  free(bo);
  return HLBG_OK;
}

void hlbo_domain_free(hlbo_domain *d) {
  free(d->nbr);
  free(d->wall_mask);
  free(d->iolet_mask);
  free(d->iolet_id);
  free(d->site_type);
  free(d->cut);
  free(d->coords);
  free(d->slot);
  memset(d, 0, sizeof(*d));
}

/* ---- initial condition --------------------------------------------------- */

void hlbo_init_equilibrium(const hlbo_domain *d, const hlbo_params *p, double rho, double ux,
                           double uy, double uz, double *f) {
  /* EquilibriumInitialCondition::SetFs (Code/lb/InitialCondition.hpp:40-52):
   * one feq(rho, rho*u) for every site */
  lat_t L;
  lattice(p->q, &L);
  double m[3] = {rho * ux, rho * uy, rho * uz};
  double feq[19];
  feq_of(&L, p->order, rho, m, feq);
  for (int64_t i = 0; i < d->n; ++i)
    for (int k = 0; k < p->q; ++k) f[i * p->q + k] = feq[k];
  f[d->n * p->q] = 0.0;
}

/* ---- one time step --------------------------------------------------------- */

static int has_bit(uint32_t mask, int dir) { return dir ? (int)((mask >> (dir - 1)) & 1u) : 0; }

static int type_of_id(const hlbo_domain *d, int64_t id) {
  int64_t acc = 0;
  for (int t = 0; t < 6; ++t) {
    acc += d->type_count[t];
    if (id < acc) return t;
  }
  return 5;
}

typedef struct {
  double in_density[4096];
} iolet_cache_unused;

/* StreamerTypeFactory::StreamAndCollide (Code/lb/streamers/StreamerTypeFactory.h:48-86)
 * with BulkLink (BulkStreamer.h:142-150), BounceBackLink (SimpleBounceBack.h:245-254),
 * BouzidiFirdaousLallemandLink (BouzidiFirdaousLallemand.h:307-334),
 * NashZerothOrderPressureLink (NashZerothOrderPressure.h:388-421) and
 * LaddIoletLink (LaddIolet.h:465-502). */
static void site_stream_collide(const lat_t *L, const hlbo_domain *d, const hlbo_params *p,
                                const double *f_old, double *f_new, uint64_t t1, int64_t i,
                                int type, const double *in_dens, const double *out_dens) {
  const int q = L->q;
  double rho, m[3], u[3], feq[19], fpost[19];
  collide(L, p, f_old + i * q, &rho, m, u, feq, fpost);
  const int can_wall = (type == 1 || type == 4 || type == 5);
  const int can_iolet = (type >= 2);
  const int is_inlet = (type == 2 || type == 4);
  const uint32_t wm = d->wall_mask[i], im = d->iolet_mask[i];
  for (int dir = 0; dir < q; ++dir) {
    if (can_iolet && has_bit(im, dir)) {
      const int bid = d->iolet_id[i];
      const int model = is_inlet ? p->inlet : p->outlet;
      const hlbg_iolet *io = is_inlet ? &p->inlets[bid] : &p->outlets[bid];
      const int unstreamed = L->inv[dir];
      if (model == HLBG_IOLET_NASH) {
        double ghost_density = is_inlet ? in_dens[bid] : out_dens[bid];
        double nd[3];
        normalise(io->normal, nd);
        /* GetNormal().as<float>() */
        float nf[3] = {(float)nd[0], (float)nd[1], (float)nd[2]};
        double nfd[3] = {(double)nf[0], (double)nf[1], (double)nf[2]};
        double component = dot3(m, nfd) / rho;
        double gm[3] = {nfd[0] * component * ghost_density, nfd[1] * component * ghost_density,
                        nfd[2] * component * ghost_density};
        double gfeq[19];
        feq_of(L, p->order, ghost_density, gm, gfeq);
        f_new[i * q + unstreamed] = gfeq[unstreamed];
      } else {
        double pos[3] = {(double)d->coords[3 * i], (double)d->coords[3 * i + 1],
                         (double)d->coords[3 * i + 2]};
        double half[3] = {pos[0] + 0.5 * L->cx[dir], pos[1] + 0.5 * L->cy[dir],
                          pos[2] + 0.5 * L->cz[dir]};
        double wallMom[3];
        /* BoundaryValues::GetTimeStep: 1-indexed, as unsigned int */
        hlbo_iolet_velocity(io, half, (uint64_t)(unsigned int)t1, wallMom);
        wallMom[0] *= rho;
        wallMom[1] *= rho;
        wallMom[2] *= rho;
        double cd[3] = {(double)L->cx[dir], (double)L->cy[dir], (double)L->cz[dir]};
        double correction = 2. * L->w[dir] * dot3(wallMom, cd) / kCs2;
        f_new[i * q + unstreamed] = fpost[dir] - correction;
      }
    } else if (can_wall && has_bit(wm, dir)) {
      const int inv = L->inv[dir];
      if (p->wall == HLBG_WALL_SBB) {
        f_new[i * q + inv] = fpost[dir];
      } else {
        double qd = d->cut[i * (q - 1) + dir - 1];
        if (has_bit(wm, inv) || qd < 0.5) {
          f_new[i * q + inv] = fpost[dir];
        } else {
          f_new[i * q + inv] = (fpost[dir] + (2.0 * qd - 1) * fpost[inv]) / (2.0 * qd);
        }
      }
    } else {
      f_new[d->nbr[i * q + dir]] = fpost[dir];
    }
  }
}

static void iolet_densities(const hlbo_params *p, uint64_t t1, double *in_d, double *out_d) {
  /* BoundaryValues::GetBoundaryDensity -> GetDensity(Get0IndexedTimeStep())
   * (Code/lb/iolets/BoundaryValues.cc:162-165, Code/lb/SimulationState.cc:44-47) */
  double mind = hlbo_min_density(p);
  for (int k = 0; k < p->n_inlets; ++k) in_d[k] = hlbo_cosine_density(&p->inlets[k], t1 - 1, mind);
  for (int k = 0; k < p->n_outlets; ++k)
    out_d[k] = hlbo_cosine_density(&p->outlets[k], t1 - 1, mind);
}

void hlbo_stream_and_collide(const hlbo_domain *d, const hlbo_params *p, const double *f_old,
                             double *f_new, uint64_t t1, int64_t first, int64_t count,
                             int n_threads) {
  lat_t L;
  lattice(p->q, &L);
  double *in_d = (double *)malloc(sizeof(double) * (p->n_inlets + 1));
  double *out_d = (double *)malloc(sizeof(double) * (p->n_outlets + 1));
  iolet_densities(p, t1, in_d, out_d);
  (void)n_threads;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(static) if (n_threads != 1)
#endif
  for (int64_t i = first; i < first + count; ++i)
    site_stream_collide(&L, d, p, f_old, f_new, t1, i, type_of_id(d, i), in_d, out_d);
  free(in_d);
  free(out_d);
}

/* StreamerTypeFactory::PostStep (StreamerTypeFactory.h:88-108) with
 * BouzidiFirdaousLallemandLink::PostStepLink (BouzidiFirdaousLallemand.h:336-357);
 * every other link streamer's PostStepLink is empty. */
void hlbo_post_step(const hlbo_domain *d, const hlbo_params *p, double *f_new, int64_t first,
                    int64_t count, int n_threads) {
  lat_t L;
  lattice(p->q, &L);
  if (p->wall != HLBG_WALL_BFL) return;
  const int q = p->q;
  (void)n_threads;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(static) if (n_threads != 1)
#endif
  for (int64_t i = first; i < first + count; ++i) {
    int type = type_of_id(d, i);
    if (!(type == 1 || type == 4 || type == 5)) continue;
    const uint32_t wm = d->wall_mask[i];
    double *fn = f_new + i * q;
    for (int dir = 0; dir < q; ++dir) {
      if (!has_bit(wm, dir)) continue;
      int inv = L.inv[dir];
      double qd = d->cut[i * (q - 1) + dir - 1];
      if (!has_bit(wm, inv) && qd < 0.5) fn[inv] = 2.0 * qd * fn[inv] + (1.0 - 2.0 * qd) * fn[dir];
    }
  }
}

void hlbo_step(const hlbo_domain *d, const hlbo_params *p, const double *f_old, double *f_new,
               uint64_t t1, int n_threads) {
  /* LBM::PreReceive over the six mid-domain ranges (Code/lb/lb.hpp:215-251); with
   * one rank there are no domain-edge sites, so PreSend has empty ranges.  Then
   * LBM::PostReceive's PostStep over the same ranges (:254-309). */
  hlbo_stream_and_collide(d, p, f_old, f_new, t1, 0, d->n, n_threads);
  hlbo_post_step(d, p, f_new, 0, d->n, n_threads);
}

void hlbo_macro(const hlbo_domain *d, const hlbo_params *p, const double *f, double *rho,
                double *u) {
  lat_t L;
  lattice(p->q, &L);
  for (int64_t i = 0; i < d->n; ++i) {
    double r, m[3];
    density_momentum(&L, p->order, f + i * p->q, &r, m);
    rho[i] = r;
    u[3 * i + 0] = m[0] / r;
    u[3 * i + 1] = m[1] / r;
    u[3 * i + 2] = m[2] / r;
  }
}

/*
 * CPU oracle for the HemeLB lattice-Boltzmann update -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's per-step LB sweep, kept to the
 * reference's data layout (AoS fOld/fNew of N*Q+1 doubles, contiguous site ids
 * ordered by collision type, int64 push table with a rubbish slot at N*Q) and to
 * its floating-point evaluation order.  Only the tests, the smoke check and the
 * CPU-baseline leg of the benchmark use it; the product never links or calls it.
 */
#ifndef HLB_ORACLE_H
#define HLB_ORACLE_H

#include <stdint.h>

#include "../include/hemelb_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic order of Lattice::CalculateDensityAndMomentum / CalculateFeq. */
#define HLBO_ORDER_SCALAR 0 /* Code/lb/lattices/Lattice.h:181-191, 332-355 (aarch64 build) */
#define HLBO_ORDER_SSE3 1   /* Code/lb/lattices/Lattice.h:119-178, 236-321 (x86_64 build) */

typedef struct hlbo_domain {
  int32_t q;
  int64_t n;              /* fluid sites */
  int64_t type_count[6];  /* contiguous ranges by collision type 0..5 */
  int64_t *nbr;           /* [n*q] push targets (Domain::neighbourIndices) */
  uint32_t *wall_mask;    /* [n] */
  uint32_t *iolet_mask;   /* [n] */
  int32_t *iolet_id;      /* [n] */
  int8_t *site_type;      /* [n] */
  double *cut;            /* [n*(q-1)] float-valued (Domain::distanceToWall) */
  int64_t *coords;        /* [n*3] global site coordinates */
  int64_t *slot;          /* [n] block_index*512 + local index in the input geometry */
} hlbo_domain;

typedef struct hlbo_params {
  int32_t q;
  int32_t kernel;  /* HLBG_KERNEL_* */
  int32_t wall;    /* HLBG_WALL_* */
  int32_t inlet;   /* HLBG_IOLET_NASH / LADD */
  int32_t outlet;
  int32_t order;   /* HLBO_ORDER_* */
  double tau;
  int32_t n_inlets, n_outlets;
  const hlbg_iolet *inlets;
  const hlbg_iolet *outlets;
} hlbo_params;

/* Build the reference Domain arrays from a sparse block geometry
 * (Domain::ProcessReadSites / PopulateWithReadData / InitialiseNeighbourLookup). */
int hlbo_domain_build(const hlbg_geometry *g, hlbo_domain *out);
void hlbo_domain_free(hlbo_domain *d);

/* Minimum iolet density over all inlets and outlets (LBM::PrepareBoundaryObjects). */
double hlbo_min_density(const hlbo_params *p);
/* InOutLetCosine::GetDensity(t). */
double hlbo_cosine_density(const hlbg_iolet *io, uint64_t t, double min_density);
/* InOutLetParabolicVelocity::GetVelocity(x, t) (and the pulsatile variant). */
void hlbo_iolet_velocity(const hlbg_iolet *io, const double x[3], uint64_t t, double out[3]);

/* Uniform equilibrium into f (EquilibriumInitialCondition::SetFs). f has n*q+1 entries. */
void hlbo_init_equilibrium(const hlbo_domain *d, const hlbo_params *p, double rho, double ux,
                           double uy, double uz, double *f);

/* One LB time step: StreamAndCollide over ranges of type 0..5, then PostStep over
 * the same ranges.  t1 = 1-indexed SimulationState time step.  The caller swaps. */
void hlbo_step(const hlbo_domain *d, const hlbo_params *p, const double *f_old, double *f_new,
               uint64_t t1, int n_threads);
/* StreamAndCollide / PostStep over [first, first+count) only (per-range streamer). */
void hlbo_stream_and_collide(const hlbo_domain *d, const hlbo_params *p, const double *f_old,
                             double *f_new, uint64_t t1, int64_t first, int64_t count,
                             int n_threads);
void hlbo_post_step(const hlbo_domain *d, const hlbo_params *p, double *f_new, int64_t first,
                    int64_t count, int n_threads);

/* Density and velocity of every site (Lattice::CalculateDensityMomentumFEq). */
void hlbo_macro(const hlbo_domain *d, const hlbo_params *p, const double *f, double *rho,
                double *u);

/* Collide one site: f[q] -> density, momentum[3], velocity[3], feq[q], fpost[q]. */
void hlbo_collide_site(const hlbo_params *p, const double *f, double *density, double *mom,
                       double *vel, double *feq, double *fpost);
/* Lattice::CalculateFeq for given density and momentum. */
void hlbo_feq(const hlbo_params *p, double density, const double mom[3], double *feq);

#ifdef __cplusplus
}
#endif
#endif

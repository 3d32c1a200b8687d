/*
 * phinum_oracle.c -- CPU restatement of PhiNum's lattice hot path.
 *
 * TEST INFRASTRUCTURE.  This file is the oracle that the GPU path is checked
 * against: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg (and its `--impl reference` arm) load it.  The product never links it
 * and never falls back to it.
 *
 * It restates, in plain C and in the reference's own operation order, the
 * functions on the path:
 *   orc_evolve           reset()/evolve()/updateMomenta()/updateFields()/
 *                        Communication::exchange()   dynamics.cpp:28-237,
 *                                                     comm.cpp:63-78
 *   orc_averages         CalculateExtrema() + CalculateVolumeAverages()
 *                                                     fieldanalysis.cpp:319-699
 *   orc_run_loop         main.cpp:685-699 with Print_AveragesExtrema()'s TSO
 *                        cadence                      fieldanalysis.cpp:748-782
 *   orc_spectrum         MomentumSpace::init/InitBCounts/
 *                        Calculate_CorrelationFunctions, fftXtoP_direct
 *                                                     momentumspace.cpp:32-278,
 *                                                     clusterfft.cpp:185-225
 *   orc_initial_conditions  SetInitialConditions (initialize 0-4, withcharge 0/1), ensureRealResult,
 *                        fftPtoX            initialconditions.cpp:14-723,
 *                                           clusterfft.cpp:10-16,55-182
 *   orc_apply_filter     apply_filter      filter.cpp:11-133
 *   orc_islands          is_island()/BFS()/Full_Analysis() scan
 *                                                     islands.cpp:72-279,778-840
 * for theories 0 (phi^4 + phi^6), 1 (phi^4 + linear h), 2 (cosine), 3
 * (cosine + monodromy mass), 4 (cubic) and 5 (power-law monodromy), static box, one
 * rank (z-slab count 1), Nc components interleaved innermost.
 *
 * Parity pin: the FP64 results are bit-identical to the reference's own
 * sources compiled by oracle/build_ref.sh (checked against the committed
 * fixtures in tests/golden/), provided this file is compiled without
 * -ffast-math and with -ffp-contract=off (GCC contracts a*b+c into FMA by
 * default on AArch64).  The spectrum uses this file's own FFT, so spectra
 * agree with the reference to rounding, and bin counts exactly.
 *
 * Layout (util.cpp:34-37, lattice.cpp:76-78): a field holds
 * Nc*N*N*(N+2) doubles, index Nc*(x + N*y + N*N*z) + a, z-slabs 0 and N+1
 * are ghosts that mirror slabs N and 1.
 */
#define _DEFAULT_SOURCE /* srand48 / drand48 under -std=c99 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "phinum_oracle.h"

/* ---------------------------------------------------------------- helpers */
static inline double sqr(double x) { return x * x; }              /* util.cpp:20-23 */
static inline int mod(int i, int n) { return i >= 0 ? i % n : (n + i) % n; } /* util.cpp:12-18 */
static inline long pos3(const orc_params *p, int x, int y, int z) {          /* util.cpp:34-37 */
  return (long)p->Nc * x + (long)p->Nc * p->N * y + (long)p->Nc * p->N * p->N * z;
}
static inline long field_len(const orc_params *p) { return (long)p->Nc * p->N * p->N * (p->N + 2); }

int orc_version(void) { return 3; }

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------ time keeping */
/* Conformal time and scale factor of the radiation-era box at cosmic time
 * tau (dynamics.cpp:39-40, :204-205). */
static void conformal(const orc_params *p, orc_clock *c) {
  c->tau_c = (sqrt(1. + 2. * p->H0 * c->tau) - 1.) / p->H0;
  c->sf = sqrt(1. + 2. * p->H0 * c->tau);
}

/* The scale factor a clock carries: 1 for the static box or no clock. */
static double clock_sf(const orc_params *p, const orc_clock *c) {
  return (p->expansion && c) ? c->sf : 1.0;
}

/* reset(): dynamics.cpp:28-50. */
void orc_reset(const orc_params *p, orc_clock *c) {
  c->tau = p->T0;
  c->dtau = p->dt * p->a;
  c->last_mom = c->tau;
  c->last_field = c->tau;
  c->steps = 0;
  c->pad_ = 0;
  if (p->expansion) {
    conformal(p, c);
  } else {
    c->tau_c = c->tau;
    c->sf = 1.0;
  }
  c->last_mom_c = c->tau_c;
  c->last_field_c = c->tau_c;
}

/* Communication::exchange() with one rank: comm.cpp:63-78. */
void orc_exchange(const orc_params *p, double *f) {
  const long slab = (long)p->Nc * p->N * p->N;
  memcpy(f + (long)(p->N + 1) * slab, f + slab, (size_t)slab * sizeof(double));
  memcpy(f, f + (long)p->N * slab, (size_t)slab * sizeof(double));
}

/* updateMomenta() of the expanding box (dynamics.cpp:88-93, :102-107,
 * :116-121, :130-135, :144-149, :158-163) at one site and component.  The
 * couplings carry powers of the scale factor sf in the reference's order of
 * operations; theories 3-5 read the a == 0 branch (they run with Nc = 1). */
static double kick_expanded(const orc_params *p, double LapPhi, double phi, double locPhiSqr, int a, double sf) {
  const int Nc = p->Nc;
  const double mass = p->m_sqr;
  switch (p->theory) {
    case 0:
      return LapPhi - ((double)p->mass_mode * mass * sf * sf + (double)p->lambda_mode * (locPhiSqr / (6. * Nc)) +
                       (sqr(locPhiSqr / p->kappa / sf) / (120. * Nc * Nc))) * phi;
    case 1:
      if (a == 0)
        return LapPhi - p->h * sf * sf * sf -
               ((double)p->mass_mode * mass * sf * sf + (double)p->lambda_mode * (locPhiSqr / (6. * Nc))) * phi;
      return LapPhi - ((double)p->mass_mode * mass * sf * sf + (double)p->lambda_mode * (locPhiSqr / (6. * Nc))) * phi;
    case 2:
      return LapPhi - mass * sqrt(mass) * sf * sf * sf * (phi / sqrt(locPhiSqr)) * sin(sqrt(locPhiSqr) / sf / sqrt(mass));
    case 3: /* the expanded monodromy force is sin(phi / (sf sqrt(M))), without the phi/|phi| factor */
      return LapPhi - p->m_mono_sqr * sf * sf * phi - mass * sqrt(mass) * sf * sf * sf * sin(phi / (sf * sqrt(mass)));
    case 4:
      return LapPhi - ((double)p->mass_mode * mass * sf * sf - p->g * sf * phi / 2. +
                       (double)p->lambda_mode * (locPhiSqr / (6. * Nc))) * phi;
    default:
      return LapPhi - mass * sf * sf * phi * pow((1. + locPhiSqr / mass / sf / sf), (p->p_mono - 1));
  }
}

/* updateMomenta(): dynamics.cpp:52-175 for theories 0 (:82-87), 1 (:96-101),
 * 2 (:109-114), 3 (:123-129), 4 (:137-143) and 5 (:151-157), slabs z in
 * [z0, z1).  sf > 0 selects the expanding box's forms (kick_expanded). */
static void update_momenta_slabs(const orc_params *p, const double *Phi, double *Pi,
                                 double factor, int z0, int z1, double sf) {
  const int N = p->N, Nc = p->Nc;
  const double mass = p->m_sqr; /* BareM_sqr_long == BareM_sqr_trans == M_sqr (renormalization.cpp:8-9) */
  for (int z = z0; z < z1; z++) {
    long Kooo = pos3(p, 0, 0, z);
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) {
        double locPhiSqr = 0.0;
        for (int a = 0; a < Nc; a++) locPhiSqr += sqr(Phi[Kooo + a]);
        long Kuoo = pos3(p, mod(x + 1, N), y, z);
        long Kouo = pos3(p, x, mod(y + 1, N), z);
        long Koou = pos3(p, x, y, z + 1);
        long Kdoo = pos3(p, mod(x - 1, N), y, z);
        long Kodo = pos3(p, x, mod(y - 1, N), z);
        long Kood = pos3(p, x, y, z - 1);
        for (int a = 0; a < Nc; a++) {
          double LapPhi = (Phi[Kuoo] + Phi[Kdoo] + Phi[Kouo] + Phi[Kodo] + Phi[Koou] + Phi[Kood] -
                           6. * Phi[Kooo]) / sqr(p->a);
          if (sf > 0) {
            Pi[Kooo] += kick_expanded(p, LapPhi, Phi[Kooo], locPhiSqr, a, sf) * factor;
          } else if (p->theory == 0) {
            Pi[Kooo] += (LapPhi - ((double)p->mass_mode * mass +
                                   (double)p->lambda_mode * (locPhiSqr / (6. * Nc)) +
                                   (sqr(locPhiSqr / p->kappa) / (120. * Nc * Nc))) * Phi[Kooo]) * factor;
          } else if (p->theory == 2) {
            Pi[Kooo] += (LapPhi - mass * sqrt(mass) * (Phi[Kooo] / sqrt(locPhiSqr)) *
                                      sin(sqrt(locPhiSqr) / sqrt(mass))) * factor;
          } else if (p->theory == 3) {
            Pi[Kooo] += (LapPhi - p->m_mono_sqr * Phi[Kooo] - mass * sqrt(mass) * (Phi[Kooo] / sqrt(locPhiSqr)) *
                                      sin(sqrt(locPhiSqr) / sqrt(mass))) * factor;
          } else if (p->theory == 4) {
            Pi[Kooo] += (LapPhi - ((double)p->mass_mode * mass - p->g * Phi[Kooo] / 2. +
                                   (double)p->lambda_mode * (locPhiSqr / (6. * Nc))) * Phi[Kooo]) * factor;
          } else if (p->theory == 5) {
            Pi[Kooo] += (LapPhi - mass * Phi[Kooo] * pow((1. + locPhiSqr / mass), (p->p_mono - 1))) * factor;
          } else {
            if (a == 0)
              Pi[Kooo] += (LapPhi - p->h - ((double)p->mass_mode * mass +
                                            (double)p->lambda_mode * (locPhiSqr / (6. * Nc))) * Phi[Kooo]) * factor;
            else
              Pi[Kooo] += (LapPhi - ((double)p->mass_mode * mass +
                                     (double)p->lambda_mode * (locPhiSqr / (6. * Nc))) * Phi[Kooo]) * factor;
          }
          Kooo++; Kuoo++; Kouo++; Koou++; Kdoo++; Kodo++; Kood++;
        }
      }
  }
}

/* evolve(): dynamics.cpp:196-237 (regime 0), nsteps times.  nthreads > 1
 * splits the z-slabs over threads like `mpirun -np K` splits them over ranks;
 * every site sees the same operations, so the result does not depend on it. */
void orc_evolve(const orc_params *p, orc_clock *c, double *Phi, double *Pi, int nsteps, int nthreads) {
  const int N = p->N;
  const long begin = pos3(p, 0, 0, 1), end = (long)p->Nc * N * N * (N + 1);
  if (nthreads < 1) nthreads = 1;
  const int ex = p->expansion;
  for (int s = 0; s < nsteps; s++) {
    c->tau += 0.5 * c->dtau;
    if (ex) conformal(p, c);
    /* the expanding box steps in conformal time (dynamics.cpp:88-93, :186-187) */
    const double fk = ex ? c->tau_c - c->last_mom_c : c->tau - c->last_mom;
    const double sf = ex ? c->sf : 0.0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
    for (int z = 1; z < N + 1; z++) update_momenta_slabs(p, Phi, Pi, fk, z, z + 1, sf);
    c->last_mom = c->tau;
    c->last_mom_c = ex ? c->tau_c : c->tau;
    c->tau += 0.5 * c->dtau;
    if (ex) conformal(p, c);
    const double fd = ex ? c->tau_c - c->last_field_c : c->tau - c->last_field;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
    for (long K = begin; K < end; K++) Phi[K] += Pi[K] * fd; /* updateFields, dynamics.cpp:180-187 */
    c->last_field = c->tau;
    c->last_field_c = ex ? c->tau_c : c->tau;
    if (!ex) {
      c->tau_c = c->tau;
      c->sf = 1.0;
    }
    orc_exchange(p, Phi);
    c->steps++;
  }
}

/* ------------------------------------------- the single-precision build */
/* With doubleprecision -1 every pseudo_double of the reference is a float
 * (parameters.cpp:13-16): the fields, the clock (dynamics.cpp:8-50), a_t,
 * M_sqr, Kappa, h, and util.cpp:20-23's sqr(), which takes and returns a
 * float.  Literals such as 6. and 120. stay double, so the kick mixes float
 * and double arithmetic by C's usual conversions, and each += rounds the
 * double sum back to float.  This restates those types for theories 0 and 1
 * on the static box. */
static inline float sqr_f(float x) { return x * x; }

void orc_reset_f32(const orc_params *p, orc_clock_f32 *c) {
  memset(c, 0, sizeof(*c));
  c->tau = (float)p->T0;                  /* LocalLattice::tau = T0 (dynamics.cpp:36) */
  c->dtau = (float)p->dt * (float)p->a;   /* dtBaseTrans * a_t, float * float (:42) */
  c->last_field = c->tau;
  c->last_mom = c->tau;
}

/* updateMomenta() theory 0 (dynamics.cpp:82-87) and 1 (:96-101), slab z. */
static void update_momenta_slab_f32(const orc_params *p, const float *Phi, float *Pi, float factor, int z) {
  const int N = p->N, Nc = p->Nc;
  const float mass = (float)p->m_sqr, kappa = (float)p->kappa, h = (float)p->h, a_t = (float)p->a;
  long Kooo = pos3(p, 0, 0, z);
  for (int y = 0; y < N; y++)
    for (int x = 0; x < N; x++) {
      float locPhiSqr = 0.0f;
      for (int a = 0; a < Nc; a++) locPhiSqr += sqr_f(Phi[Kooo + a]);
      long Kuoo = pos3(p, mod(x + 1, N), y, z);
      long Kouo = pos3(p, x, mod(y + 1, N), z);
      long Koou = pos3(p, x, y, z + 1);
      long Kdoo = pos3(p, mod(x - 1, N), y, z);
      long Kodo = pos3(p, x, mod(y - 1, N), z);
      long Kood = pos3(p, x, y, z - 1);
      for (int a = 0; a < Nc; a++) {
        /* the six float additions, then a double subtraction and division */
        float LapPhi = (float)((Phi[Kuoo] + Phi[Kdoo] + Phi[Kouo] + Phi[Kodo] + Phi[Koou] + Phi[Kood] -
                                6. * Phi[Kooo]) / sqr_f(a_t));
        double f;
        if (p->theory == 0)
          f = LapPhi - (p->mass_mode * mass + p->lambda_mode * (locPhiSqr / (6. * Nc)) +
                        (sqr_f(locPhiSqr / kappa) / (120. * Nc * Nc))) * Phi[Kooo];
        else if (a == 0)
          f = (LapPhi - h) - (p->mass_mode * mass + p->lambda_mode * (locPhiSqr / (6. * Nc))) * Phi[Kooo];
        else
          f = LapPhi - (p->mass_mode * mass + p->lambda_mode * (locPhiSqr / (6. * Nc))) * Phi[Kooo];
        Pi[Kooo] = (float)(Pi[Kooo] + f * factor);
        Kooo++; Kuoo++; Kouo++; Koou++; Kdoo++; Kodo++; Kood++;
      }
    }
}

/* evolve() (dynamics.cpp:196-237) in the single-precision build. */
void orc_evolve_f32(const orc_params *p, orc_clock_f32 *c, float *Phi, float *Pi, int nsteps, int nthreads) {
  const int N = p->N;
  const long slab = (long)p->Nc * N * N;
  const long begin = slab, end = slab * (N + 1);
  if (nthreads < 1) nthreads = 1;
  (void)nthreads;
  for (int s = 0; s < nsteps; s++) {
    c->tau = (float)(c->tau + 0.5 * c->dtau);
    const float fk = c->tau - c->last_mom;  /* tau - Last_Momenta_update, float */
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
    for (int z = 1; z < N + 1; z++) update_momenta_slab_f32(p, Phi, Pi, fk, z);
    c->last_mom = c->tau;
    c->tau = (float)(c->tau + 0.5 * c->dtau);
    const float fd = c->tau - c->last_field;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
    for (long K = begin; K < end; K++) Phi[K] += Pi[K] * fd; /* updateFields, dynamics.cpp:180-183 */
    c->last_field = c->tau;
    memcpy(Phi + (long)(N + 1) * slab, Phi + slab, (size_t)slab * sizeof(float)); /* exchange, comm.cpp:63-78 */
    memcpy(Phi, Phi + (long)N * slab, (size_t)slab * sizeof(float));
    c->steps++;
  }
}

/* ---------------------------------------------------------------- averages */
/* CalculateExtrema(): fieldanalysis.cpp:319-397 (one rank). */
static void extrema(const orc_params *p, const double *Phi, orc_row *o) {
  const int Nc = p->Nc, N = p->N;
  double maxPhi = -10000000.0, minPhi = 10000000.0, maxAbsPhi = 0.0;
  long maxpos = -1, minpos = -1, maxAbspos = -1;
  double AbsPhi = 0.;
  for (long k = pos3(p, 0, 0, 1); k < (long)Nc * N * N * (N + 1); k++) {
    AbsPhi += ((Phi[k]) * (Phi[k]));
    if ((k + 1) % Nc == 0) {
      AbsPhi = sqrt(AbsPhi);
      if (AbsPhi > maxAbsPhi) {
        maxAbsPhi = AbsPhi;
        maxAbspos = k + 1 - Nc;
      }
      AbsPhi = 0;
    }
    if (Phi[k] > maxPhi) { maxPhi = Phi[k]; maxpos = k; }
    if (Phi[k] < minPhi) { minPhi = Phi[k]; minpos = k; }
  }
  o->min_phi = minPhi;
  o->max_phi = maxPhi;
  o->max_abs_phi = maxAbsPhi;
  o->min_pos = (double)minpos;
  o->max_pos = (double)maxpos;
  o->max_abs_pos = (double)maxAbspos;
}

/* The per-site (all components) interaction terms of CalculateVolumeAverages
 * (fieldanalysis.cpp:565-617; per component :456-508), static box; locPhi is the sum of the
 * components (:434-443). */
static double site_interaction(const orc_params *p, double locPhiSqr, double locPhi, double sf) {
  const int Nc = p->Nc;
  const double mass = p->m_sqr;
  if (p->expansion) /* fieldanalysis.cpp:573-615 */
    switch (p->theory) {
      case 0:
        return ((double)(p->lambda_mode) * (sqr(locPhiSqr) / (24.0 * Nc)) +
                (sqr(locPhiSqr) * locPhiSqr / (720.0 * Nc * Nc * p->kappa * p->kappa * sf * sf)));
      case 1:
        return (double)(p->lambda_mode) * (sqr(locPhiSqr) / (24.0 * Nc));
      case 2:
      case 3:
        return sqr(sf * sf * mass) * (1. - cos(sqrt(locPhiSqr) / (sf * sqrt(mass))));
      case 4:
        return (((-p->g * sf * locPhi * locPhiSqr) / (6.0)) + (double)(p->lambda_mode) * (sqr(locPhiSqr) / (24.0 * Nc)));
      default:
        return sqr(sf * sf * mass) * 0.5 / p->p_mono * (pow((1. + locPhiSqr / mass / sf / sf), p->p_mono) - 1.);
    }
  switch (p->theory) {
    case 0:
      return (double)(p->lambda_mode) * (sqr(locPhiSqr) / (24.0 * Nc)) +
             (sqr(locPhiSqr) * locPhiSqr / (720.0 * Nc * Nc * p->kappa * p->kappa));
    case 1:
      return (double)(p->lambda_mode) * (sqr(locPhiSqr) / (24.0 * Nc));
    case 2:
    case 3:
      return sqr(mass) * (1. - cos(sqrt(locPhiSqr / mass)));
    case 4:
      return (((-p->g * locPhi * locPhiSqr) / (6.0)) + (double)(p->lambda_mode) * (sqr(locPhiSqr) / (24.0 * Nc)));
    default:
      return sqr(mass) * 0.5 / p->p_mono * (pow((1. + locPhiSqr / mass), p->p_mono) - 1.);
  }
}

/* The per-component mass / linear terms of CalculateVolumeAverages
 * (fieldanalysis.cpp:454-508): static box, or expanding box with scale
 * factor sf. */
static double component_interaction(const orc_params *p, double phi, int a, double sf) {
  const double mass = p->m_sqr;
  if (p->expansion) {
    if (p->theory == 0 || p->theory == 4)
      return (double)(p->mass_mode) * 0.5 * mass * sf * sf * sqr(phi);
    if (p->theory == 3)
      return (0.5 * p->m_mono_sqr * (sqr(sf)) * sqr(phi));
    if (p->theory == 1 && a == 0)
      return (p->h * phi * sf * sf * sf + (double)(p->mass_mode) * 0.5 * mass * sf * sf * sqr(phi));
    if (p->theory == 1)
      return (double)(p->mass_mode) * 0.5 * mass * sf * sf * sqr(phi);
    return 0.0;
  }
  if (p->theory == 0 || p->theory == 4)
    return (double)(p->mass_mode) * 0.5 * mass * sqr(phi);
  if (p->theory == 3)
    return 0.5 * p->m_mono_sqr * sqr(phi);
  if (p->theory == 1 && a == 0)
    return (p->h * phi + (double)(p->mass_mode) * 0.5 * mass * sqr(phi));
  if (p->theory == 1)
    return (double)(p->mass_mode) * 0.5 * mass * sqr(phi);
  return 0.0;
}

/* CalculateVolumeAverages(): fieldanalysis.cpp:399-699, theories 0 to 5,
 * static or expanding box (scale factor sf), no charge / energy-density
 * extras.  Also returns the gradient term GradPhiSqr/vol, which the
 * reference keeps local. */
static void volume_averages(const orc_params *p, const double *Phi, const double *Pi, orc_row *o, double sf) {
  const int N = p->N, Nc = p->Nc;
  const int vol = N * N * N;
  double phi[ORC_MAX_NC], pi[ORC_MAX_NC];
  for (int a = 0; a < Nc; a++) { phi[a] = 0.0; pi[a] = 0.0; }
  double phi2 = 0., pi2 = 0., phi4 = 0., phi6 = 0., phipi = 0.;
  double Interaction = 0., Charge = 0., Energy;
  double GradPhiSqr = 0.0;
  long Kooo = pos3(p, 0, 0, 1);
  for (int z = 1; z < N + 1; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) {
        long Kuoo = pos3(p, mod(x + 1, N), y, z);
        long Kouo = pos3(p, x, mod(y + 1, N), z);
        long Koou = pos3(p, x, y, z + 1);
        double locPhiSqr = 0.0;
        double locPhi = 0.;
        for (int a = 0; a < Nc; a++) {
          phi[a] += Phi[Kooo]; pi[a] += Pi[Kooo];
          phi2 += sqr(Phi[Kooo]); pi2 += sqr(Pi[Kooo]);
          phipi += Phi[Kooo] * Pi[Kooo];
          locPhiSqr += sqr(Phi[Kooo]);
          locPhi += Phi[Kooo];
          GradPhiSqr += (sqr(Phi[Kuoo] - Phi[Kooo]) / sqr(p->a) + sqr(Phi[Kouo] - Phi[Kooo]) / sqr(p->a) +
                         sqr(Phi[Koou] - Phi[Kooo]) / sqr(p->a));
          if (p->theory == 0 || p->theory == 1 || p->theory == 3 || p->theory == 4)
            Interaction += component_interaction(p, Phi[Kooo], a, sf);
          Kooo++; Kuoo++; Kouo++; Koou++;
        }
        phi4 += sqr(locPhiSqr);
        phi6 += sqr(locPhiSqr) * locPhiSqr;
        Interaction += site_interaction(p, locPhiSqr, locPhi, sf);
      }
  for (int a = 0; a < Nc; a++) { phi[a] /= (vol); pi[a] /= (vol); }
  Charge = (0.5 * pi2 - GradPhiSqr / 6. - Interaction);
  Energy = (0.5 * pi2 + 0.5 * GradPhiSqr + Interaction);
  if (p->expansion) { /* fieldanalysis.cpp:626-629 */
    Energy += (0.5 * phi2 * sqr(p->H0 / sf) - phipi * p->H0 / sf);
    Charge += (0.5 * phi2 * sqr(p->H0 / sf) - phipi * p->H0 / sf);
  }
  Energy /= (vol);
  Interaction /= (vol);
  Charge /= (vol);
  phi2 /= (vol); pi2 /= (vol);
  phi4 /= (vol);
  phi6 /= (vol);
  phipi /= (vol);
  /* MPI_Reduce + "/nodes" with one rank (fieldanalysis.cpp:658-685) is the identity */
  for (int a = 0; a < ORC_MAX_NC; a++) {
    o->phi[a] = a < Nc ? phi[a] : 0.0;
    o->pi[a] = a < Nc ? pi[a] : 0.0;
  }
  o->phi2 = phi2; o->pi2 = pi2; o->phipi = phipi; o->phi4 = phi4; o->phi6 = phi6;
  o->energy = Energy; o->interaction = Interaction; o->charge = Charge;
  o->gradient = GradPhiSqr / (vol);
}

void orc_averages(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi, orc_row *o) {
  memset(o, 0, sizeof(*o));
  o->t = c ? c->tau : 0.0;
  extrema(p, Phi, o);
  const double sf = clock_sf(p, c);
  volume_averages(p, Phi, Pi, o, sf);
  o->reserved[1] = sf; /* the SO row's scale factor (fieldanalysis.cpp:789-791); 1 for the static box */
}

/* main.cpp:685-699 with an explicit step count; Print_AveragesExtrema()'s
 * cadence (fieldanalysis.cpp:753-780): a row at step 0, then whenever
 * tau >= LastSO + TSO, where LastSO advances by TSO.  Rows are stamped with
 * LastSO, the time the reference prints.  Returns the number of rows. */
int orc_run_loop(const orc_params *p, orc_clock *c, double *Phi, double *Pi, int nsteps, double tso,
                 orc_row *rows, int max_rows, int nthreads) {
  int nrows = 0;
  double last_so = 0.0;
  orc_reset(p, c);
  for (int count = 0; count < nsteps; count++) {
    int due = 0;
    if (c->steps == 0) {
      last_so = c->tau;
      due = 1;
    } else if (!(c->tau < last_so + tso)) {
      if (c->tau >= last_so + tso) last_so += tso;
      due = 1;
    }
    if (due && nrows < max_rows) {
      orc_averages(p, c, Phi, Pi, &rows[nrows]);
      rows[nrows].t = last_so;
      nrows++;
    }
    orc_evolve(p, c, Phi, Pi, 1, nthreads);
  }
  return nrows;
}

/* ---------------------------------------------------------------- spectrum */
/* MomentumSpace::init (momentumspace.cpp:32-47): bin width and count. */
void orc_spectrum_bins(const orc_params *p, int *nbins, double *binsize) {
  double pTmin = (2.0 / (p->a)) * sin(acos(-1.) / p->N);
  double pTmax = sqrt(3.0 * (4.0 / sqr(p->a)));
  *binsize = pTmin;
  *nbins = (int)(pTmax / pTmin + 0.5) + 2;
}

/* Lattice momentum along one axis for index n (momentumspace.cpp:222-235,
 * the halved axis at :244 uses the positive branch only). */
static double lattice_p(int n, int N, double a) {
  if (n < N / 2 + 1) return 2.0 / (a) * sin(n * acos(-1.) / N);
  return -2.0 / (a) * sin(n * acos(-1.) / N);
}

/* In-place complex DFT of length n with stride; radix-2 when n is a power of
 * two, direct sum otherwise.  sign = -1 is the forward transform. */
static void dft_line(double *re, double *im, int n, long stride, double *wr, double *wi) {
  if (n <= 1) return;
  const double two_pi = 6.283185307179586476925286766559;
  if ((n & (n - 1)) == 0) {
    for (int i = 1, j = 0; i < n; i++) {
      int bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) {
        double t = re[i * stride]; re[i * stride] = re[j * stride]; re[j * stride] = t;
        t = im[i * stride]; im[i * stride] = im[j * stride]; im[j * stride] = t;
      }
    }
    for (int len = 2; len <= n; len <<= 1) {
      int half = len >> 1;
      for (int k = 0; k < half; k++) {
        double ang = two_pi * (double)k / (double)len;
        double cr = cos(ang), ci = -sin(ang);
        for (int s = 0; s < n; s += len) {
          long i0 = (long)(s + k) * stride, i1 = (long)(s + k + half) * stride;
          double br = re[i1] * cr - im[i1] * ci;
          double bi = re[i1] * ci + im[i1] * cr;
          re[i1] = re[i0] - br; im[i1] = im[i0] - bi;
          re[i0] += br; im[i0] += bi;
        }
      }
    }
    return;
  }
  for (int k = 0; k < n; k++) {
    double sr = 0, si = 0;
    for (int j = 0; j < n; j++) {
      double ang = two_pi * (double)((long)k * j % n) / (double)n;
      double cr = cos(ang), ci = -sin(ang);
      sr += re[j * stride] * cr - im[j * stride] * ci;
      si += re[j * stride] * ci + im[j * stride] * cr;
    }
    wr[k] = sr; wi[k] = si;
  }
  for (int k = 0; k < n; k++) { re[k * stride] = wr[k]; im[k * stride] = wi[k]; }
}

/* 3-D forward DFT of component `comp` of a field, scaled by a^3
 * (fftXtoP_direct, clusterfft.cpp:185-225).  Output is the full complex
 * spectrum, index kx + N*ky + N*N*kz. */
static void forward_fft(const orc_params *p, const double *f, int comp, double *re, double *im) {
  const int N = p->N;
  const long NN = (long)N * N;
  double *wr = (double *)malloc(sizeof(double) * N), *wi = (double *)malloc(sizeof(double) * N);
  for (int z = 0; z < N; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) {
        re[x + N * y + NN * z] = f[comp + pos3(p, x, y, z + 1)];
        im[x + N * y + NN * z] = 0.0;
      }
  for (long r = 0; r < NN; r++) dft_line(re + r * N, im + r * N, N, 1, wr, wi);
  for (int z = 0; z < N; z++)
    for (int x = 0; x < N; x++) dft_line(re + x + NN * z, im + x + NN * z, N, N, wr, wi);
  for (long r = 0; r < NN; r++) dft_line(re + r, im + r, N, NN, wr, wi);
  const double factor = (sqr(p->a) * p->a);
  for (long i = 0; i < NN * N; i++) { re[i] *= factor; im[i] *= factor; }
  free(wr); free(wi);
}

/* InitBCounts + Calculate_CorrelationFunctions (momentumspace.cpp:89-278):
 * F/K/Q[bin*Nc + a] = sum over modes px, pz in [0,N), py in [0,N/2] of
 * |Phi_p|^2, |Pi_p|^2, Re(Phi_p conj Pi_p), each counted twice unless py is 0
 * or N/2; counts[bin] likewise.  py runs over lattice y (the reference's
 * transposed FFT input puts y on the halved axis, clusterfft.cpp:198). */
int orc_spectrum(const orc_params *p, const double *Phi, const double *Pi, double *F, double *K, double *Q,
                 int *counts) {
  const int N = p->N, Nc = p->Nc;
  int nb;
  double binsize;
  orc_spectrum_bins(p, &nb, &binsize);
  const long NN = (long)N * N, V = NN * N;
  for (int k = 0; k < nb * Nc; k++) { F[k] = 0.; K[k] = 0.; Q[k] = 0.; }
  for (int k = 0; k < nb; k++) counts[k] = 0;
  double *fr = (double *)malloc(sizeof(double) * V), *fi = (double *)malloc(sizeof(double) * V);
  double *gr = (double *)malloc(sizeof(double) * V), *gi = (double *)malloc(sizeof(double) * V);
  int bad = 0;
  for (int a = 0; a < Nc; a++) {
    forward_fft(p, Phi, a, fr, fi);
    forward_fft(p, Pi, a, gr, gi);
    for (int pz = 0; pz < N; pz++) {
      double nu = (pz == 0) ? 0 : lattice_p(pz, N, p->a);
      for (int px = 0; px < N; px++) {
        double ppx = lattice_p(px, N, p->a);
        for (int py = 0; py < N / 2 + 1; py++) {
          double ppy = 2.0 / (p->a) * sin(py * acos(-1.) / N);
          double psqr = sqr(ppx) + sqr(ppy) + sqr(nu);
          int bin = (int)(sqrt(psqr) / binsize + 0.5);
          if (bin >= nb) { bad = 1; continue; }
          long m = px + (long)N * py + NN * pz;
          double af = hypot(fr[m], fi[m]), ak = hypot(gr[m], gi[m]);
          double q = fr[m] * gr[m] + fi[m] * gi[m];
          int w = (py != 0 && py != N / 2) ? 2 : 1;
          for (int r = 0; r < w; r++) {
            F[bin * Nc + a] += sqr(af);
            K[bin * Nc + a] += sqr(ak);
            Q[bin * Nc + a] += q;
            if (a == 0) counts[bin]++;
          }
        }
      }
    }
  }
  free(fr); free(fi); free(gr); free(gi);
  return bad ? -1 : nb;
}

/* Config-mode spectrum (the configuration's radial |k| bins; no reference
 * counterpart): the modes, weights and sums of orc_spectrum, binned
 * uniformly in the lattice momentum |p| on [0, p_max], p_max = pTmax of
 * momentumspace.cpp:43 (the largest |p|): bin = (int)(|p| / (p_max / nbins)),
 * the top edge folded into the last bin.  Returns nbins. */
int orc_spectrum_uniform(const orc_params *p, const double *Phi, const double *Pi, int nbins, double *F, double *K,
                         double *Q, int *counts) {
  const int N = p->N, Nc = p->Nc;
  const double pmax = sqrt(3.0 * (4.0 / sqr(p->a)));
  const double width = pmax / nbins;
  const long NN = (long)N * N, V = NN * N;
  for (int k = 0; k < nbins * Nc; k++) { F[k] = 0.; K[k] = 0.; Q[k] = 0.; }
  for (int k = 0; k < nbins; k++) counts[k] = 0;
  double *fr = (double *)malloc(sizeof(double) * V), *fi = (double *)malloc(sizeof(double) * V);
  double *gr = (double *)malloc(sizeof(double) * V), *gi = (double *)malloc(sizeof(double) * V);
  for (int a = 0; a < Nc; a++) {
    forward_fft(p, Phi, a, fr, fi);
    forward_fft(p, Pi, a, gr, gi);
    for (int pz = 0; pz < N; pz++) {
      double nu = lattice_p(pz, N, p->a);
      for (int px = 0; px < N; px++) {
        double ppx = lattice_p(px, N, p->a);
        for (int py = 0; py < N / 2 + 1; py++) {
          double ppy = lattice_p(py, N, p->a);
          double psqr = sqr(ppx) + sqr(ppy) + sqr(nu);
          int bin = (int)(sqrt(psqr) / width);
          if (bin >= nbins) bin = nbins - 1;
          long m = px + (long)N * py + NN * pz;
          double f = sqr(fr[m]) + sqr(fi[m]), k = sqr(gr[m]) + sqr(gi[m]);
          double q = fr[m] * gr[m] + fi[m] * gi[m];
          int w = (py != 0 && py != N / 2) ? 2 : 1;
          F[bin * Nc + a] += w * f;
          K[bin * Nc + a] += w * k;
          Q[bin * Nc + a] += w * q;
          if (a == 0) counts[bin] += w;
        }
      }
    }
  }
  free(fr); free(fi); free(gr); free(gi);
  return nbins;
}

/* ------------------------------------------------------ initial conditions */
/* randGen::Gauss (initialconditions.cpp:27-41): polar Box-Muller on drand48,
 * the second value cached for the next call. */
static int ic_on = 0;
static double ic_gauss2 = 0.0;
static double ic_gauss(void) {
  if (ic_on == 1) { ic_on = 0; return ic_gauss2; }
  double x, y, r, c, s, g1;
  int accept = 0;
  while (accept == 0) {
    x = 2.0 * drand48() - 1.0; y = 2.0 * drand48() - 1.0;
    r = sqrt(sqr(x) + sqr(y));
    if (r < 1.0) accept = 1;
  }
  c = x / r; s = y / r;
  g1 = c * sqrt(-2.0 * log(sqr(r)));
  ic_gauss2 = (s / c) * g1;
  ic_on = 1;
  return g1;
}

/* sgn of clusterfft.cpp:10-16 (sgn(0) = -1). */
static int ic_sgn(double x) { return x > 0 ? 1 : -1; }

/* ensureRealResult (clusterfft.cpp:55-139) for one rank: F[py + px M + pz N M]. */
static void ic_ensure_real(int N, double *re, double *im) {
  const int M = N / 2 + 1;
  for (int pz = 0; pz < N; pz++)
    for (int px = 0; px < N; px++)
      for (int py = 0; py < M; py++) {
        const int mpz = mod(N - pz, N), mpx = mod(N - px, N), mpy = mod(N - py, N);
        if (mpy != py) continue;
        const long i = py + (long)px * M + (long)pz * N * M;
        if (px == mpx && pz == mpz) {
          const double v = hypot(re[i], im[i]) * ic_sgn(re[i]);
          re[i] = v; im[i] = 0.0;
        } else {
          const long j = mpy + (long)mpx * M + (long)mpz * N * M;
          re[j] = re[i]; im[j] = -im[i];
        }
      }
}

/* fftPtoX (clusterfft.cpp:148-182): the half spectrum [pz][px][py] is
 * completed by Hermitian symmetry and transformed with exp(+2 pi i ...);
 * out[x + N y + N^2 z] = X(z, x, y) / L^3.  The inverse transform is the
 * conjugate of the forward transform of the conjugate. */
static void ic_fft_ptox(const orc_params *p, const double *hre, const double *him, double *out) {
  const int N = p->N, M = N / 2 + 1;
  const long NN = (long)N * N, V = NN * N;
  double *re = (double *)malloc(sizeof(double) * V), *im = (double *)malloc(sizeof(double) * V);
  double *wr = (double *)malloc(sizeof(double) * N), *wi = (double *)malloc(sizeof(double) * N);
  /* full[py + N px + N^2 pz] */
  for (int pz = 0; pz < N; pz++)
    for (int px = 0; px < N; px++)
      for (int py = 0; py < N; py++) {
        double vr, vi;
        if (py < M) {
          const long i = py + (long)px * M + (long)pz * N * M;
          vr = hre[i]; vi = him[i];
        } else {
          const long i = (N - py) + (long)mod(N - px, N) * M + (long)mod(N - pz, N) * N * M;
          vr = hre[i]; vi = -him[i];
        }
        re[py + N * px + NN * pz] = vr;
        im[py + N * px + NN * pz] = -vi; /* conjugate in */
      }
  for (long r = 0; r < NN; r++) dft_line(re + r * N, im + r * N, N, 1, wr, wi);
  for (int z = 0; z < N; z++)
    for (int y = 0; y < N; y++) dft_line(re + y + NN * z, im + y + NN * z, N, N, wr, wi);
  for (long r = 0; r < NN; r++) dft_line(re + r, im + r, N, NN, wr, wi);
  const double Norm = sqr(p->a * N) * N * p->a;
  /* conjugate out: the real part is unchanged; re[y + N x + N^2 z] = X(z, x, y) */
  for (int z = 0; z < N; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) out[x + N * y + NN * z] = re[y + N * x + NN * z] / Norm;
  free(re); free(im); free(wr); free(wi);
}

/* SetInitialConditions (initialconditions.cpp:45-723), initialize 3,
 * withcharge 0, one rank.  The expanding box (:459-465, :504-510, :581-583,
 * :656-658) seeds a scale-invariant spectrum below QS, frequencies with the
 * initial scale factor squared, E = H0 A and Pi_0 += phi0_0 H0.  Phi/Pi in
 * the reference layout; Phi's ghost slabs exchanged, Pi's left as they
 * were.  Returns 0. */
/* Occupation and Omega of one mode and component (initialconditions.cpp):
 * the withcharge 0 branches (:308-508) or the withcharge 1 ones (:160-257),
 * each with its own comparisons; the expanding box's forms belong to
 * initialize 3 without charge.  Returns 0, or -1 for initialize 4 with
 * charge, where the reference sets neither. */
static int ic_occupation(const orc_params *p, const orc_ic *ic, int a, double pt, double nu, double psqr,
                         double *occ, double *omega) {
  const int Nc = p->Nc;
  const double M = p->m_sqr;
  double pchisqr;
  switch (ic->initialize) {
    case 0: /* parametric resonance (:163-175, :310-321) */
      if (a == 0) *omega = sqrt(psqr + fabs(M) - 3. * sqr(ic->temperature) * sqr(ic->phi0s) / (6. * Nc));
      else *omega = sqrt(psqr + fabs(M) - sqr(ic->temperature) * sqr(ic->phi0s) / (6. * Nc));
      *occ = ic->famp * ic->lambda;
      return 0;
    case 1: /* box (:180-206, :326-350) */
      pchisqr = sqr(pt) + sqr(ic->chi) * sqr(nu);
      if (sqrt(pchisqr) < ic->QS) *occ = ic->amplitude;
      else *occ = sqrt(pchisqr) < 2.0 * ic->QS ? ic->noise : 0.0;
      break;
    case 2: /* large-Lambda box (:211-251, :357-397) */
      pchisqr = sqr(pt) + sqr(nu);
      if (ic->justnoise == 0 && sqrt(pchisqr) < ic->QS) *occ = ic->amplitude + ic->noise;
      else if (ic->scale2 == 0) *occ = ic->noise;
      else *occ = sqrt(pchisqr) < ic->scale2 ? ic->noise : 0.0;
      break;
    case 3:
      pchisqr = sqr(pt) + sqr(nu);
      if (ic->withcharge) { /* :255-291: static forms only */
        if (ic->justnoise == 0 && sqrt(pchisqr) < ic->QS) *occ = ic->amplitude + ic->noise;
        else if (ic->scale2 == 0) *occ = ic->noise;
        else *occ = sqrt(pchisqr) < ic->scale2 ? ic->noise : 0.0;
        *omega = a == 0 ? sqrt(psqr + ic->m2_long) : sqrt(psqr + ic->m2_trans);
        return 0;
      }
      /* :402-510 */
      if (ic->justnoise == 0 && p->expansion && psqr > 0. && psqr < (ic->QS * ic->QS)) {
        const double omegap = sqrt(psqr + (1. + 2. * p->H0 * p->T0) * ic->m2_long);
        *occ = 2. * acos(-1.) * acos(-1.) * 2.1e-9 * ic->phi0[0] * ic->phi0[0] / psqr / sqrt(psqr) * omegap;
      } else if (ic->justnoise == 0 && !p->expansion && pchisqr < ic->QS * ic->QS) {
        *occ = ic->amplitude + ic->noise;
      } else {
        if (ic->scale2 == 0) *occ = ic->noise;
        else *occ = sqrt(pchisqr) < ic->scale2 ? ic->noise : 0.0;
      }
      {
        const double m2 = a == 0 ? ic->m2_long : ic->m2_trans;
        *omega = p->expansion ? sqrt(psqr + (1. + 2. * p->H0 * p->T0) * m2) : sqrt(psqr + m2);
      }
      return 0;
    case 4: /* :514-556, no charged form */
      if (ic->withcharge) return -1;
      pchisqr = sqr(pt) + sqr(nu);
      if (ic->justnoise == 0 && pchisqr < ic->QS * ic->QS) *occ = ic->temperature / sqrt(psqr + ic->m2_long) + ic->noise;
      else if (ic->scale2 == 0) *occ = ic->noise;
      else *occ = sqrt(pchisqr) < ic->scale2 ? ic->noise : 0.0;
      *omega = a == 0 ? sqrt(psqr + ic->m2_long) : sqrt(psqr + ic->m2_trans);
      return 0;
    default:
      return -1;
  }
  /* initialize 1 and 2 (:197-204, :244-249, :343-350, :390-397) */
  if (a == 0) *omega = sqrt(psqr + fabs(M) - 3. * sqr(ic->phi0s) / (6. * Nc));
  else *omega = sqrt(psqr + fabs(M) - sqr(ic->phi0s) / (6. * Nc));
  return 0;
}

/* SetInitialConditions (initialconditions.cpp:45-723) for initialize 0-4,
 * withcharge 0 or 1, static or expanding box.  Per mode (pz, px, py <= N/2)
 * and component: two phases and two |Gaussians| -- except with charge and
 * Nc = 2 (:132-147), where component 0 takes nothing new and component 1
 * shifts the previous phase and Gaussian into phase2/gauss2 and draws one of
 * each, so component 0 of a mode uses component 1's draws of the two modes
 * before it.  Those are uninitialized locals for the first mode (:72-76);
 * the reference pin reads them as 0, and so does this restatement. */
int orc_initial_conditions(const orc_params *p, const orc_ic *ic, double *Phi, double *Pi) {
  const int N = p->N, Nc = p->Nc, M = N / 2 + 1;
  const long NM = (long)N * N * M, NN = (long)N * N;
  const double a = p->a;
  if (ic->initialize < 0 || ic->initialize > 4 || (ic->initialize == 4 && ic->withcharge)) return -1;
  double *Are = (double *)calloc((size_t)Nc * NM, sizeof(double)), *Aim = (double *)calloc((size_t)Nc * NM, sizeof(double));
  double *Ere = (double *)calloc((size_t)Nc * NM, sizeof(double)), *Eim = (double *)calloc((size_t)Nc * NM, sizeof(double));
  double *X = (double *)malloc(sizeof(double) * NN * N);
  const int paired = ic->withcharge && Nc == 2;
  double phase1 = 0.0, phase2 = 0.0, gauss1 = 0.0, gauss2 = 0.0;
  srand48(ic->seed);
  ic_on = 0;
  for (int pz = 0; pz < N; pz++) {
    double nu;
    if (pz == 0) nu = 0;
    else if (pz < N / 2 + 1) nu = 2.0 / (a) * sin((pz) * acos(-1.) / N);
    else nu = -2.0 / (a) * sin((pz) * acos(-1.) / N);
    for (int px = 0; px < N; px++) {
      double ppx;
      if (px < N / 2 + 1) ppx = 2.0 / (a) * sin(px * acos(-1.) / N);
      else ppx = -2.0 / (a) * sin(px * acos(-1.) / N);
      for (int py = 0; py < M; py++) {
        const double ppy = 2.0 / (a) * sin(py * acos(-1.) / N);
        const double pt = sqrt(sqr(ppx) + sqr(ppy));
        const double psqr = sqr(pt) + sqr(nu);
        const long posMom = py + (long)px * M + (long)pz * N * M;
        for (int c = 0; c < Nc; c++) {
          if (paired) {
            if (c == 1) {
              phase2 = phase1;
              phase1 = 2.0 * acos(-1.) * drand48();
              gauss2 = gauss1;
              gauss1 = fabs(ic_gauss());
            }
          } else {
            phase1 = 2.0 * acos(-1.) * drand48();
            phase2 = 2.0 * acos(-1.) * drand48();
            gauss1 = fabs(ic_gauss());
            gauss2 = fabs(ic_gauss());
          }
          double occ = 0.0, omega = 0.0;
          ic_occupation(p, ic, c, pt, nu, psqr, &occ, &omega);
          const double s1 = sqrt(occ) * gauss1, s2 = sqrt(occ) * gauss2;
          const long o = (long)c * NM + posMom;
          if (fabs(omega) < 1e-8) {
            Are[o] = Aim[o] = Ere[o] = Eim[o] = 0.0;
          } else {
            const double so = sqrt(omega);
            Are[o] = s1 * cos(phase1) / so; Aim[o] = s1 * sin(phase1) / so;
            if (p->expansion && !ic->withcharge) { /* E = A H_0 (:581-583) */
              Ere[o] = Are[o] * p->H0; Eim[o] = Aim[o] * p->H0;
            } else {
              Ere[o] = s2 * cos(phase2) * so; Eim[o] = s2 * sin(phase2) * so;
            }
          }
        }
      }
    }
  }
  const double NormFactor = sqrt(sqr(N * a) * N * a);
  for (int c = 0; c < Nc; c++) {
    ic_ensure_real(N, Are + (long)c * NM, Aim + (long)c * NM);
    ic_ensure_real(N, Ere + (long)c * NM, Eim + (long)c * NM);
  }
  /* the lattice values (:634-690): initialize 3 and 4 add phi0_0/1, pi0_0/1
   * (+ phi0_0 H_0 to Pi's component 0 in the expanding box), the others
   * phi0, pi0 to component 0 only */
  const int own = ic->initialize == 3 || ic->initialize == 4;
  for (int f = 0; f < 2; f++)
    for (int c = 0; c < Nc; c++) {
      ic_fft_ptox(p, (f == 0 ? Are : Ere) + (long)c * NM, (f == 0 ? Aim : Eim) + (long)c * NM, X);
      double off;
      if (own) off = c < 2 ? (f == 0 ? ic->phi0[c] : ic->pi0[c]) : 0.0;
      else off = c == 0 ? (f == 0 ? ic->phi0s : ic->pi0s) : 0.0;
      const int hubble = own && p->expansion && f == 1 && c == 0; /* + phi0_0 H0 (:657) */
      double *dst = f == 0 ? Phi : Pi;
      for (int z = 0; z < N; z++)
        for (int y = 0; y < N; y++)
          for (int x = 0; x < N; x++) {
            const double v = X[x + N * y + NN * z] * NormFactor + off;
            dst[c + pos3(p, x, y, z + 1)] = hubble ? v + ic->phi0[0] * p->H0 : v;
          }
    }
  orc_exchange(p, Phi); /* Communication::exchange moves Phi only (comm.cpp:63-78) */
  free(Are); free(Aim); free(Ere); free(Eim); free(X);
  return 0;
}

/* ------------------------------------------------------- momentum filter */
/* Window functions of filter.cpp:11-51. */
static double flt_w(int which, double r, double p, const double *table, int ntable, double dp) {
  if (which == 0) {
    if (p * r == 0) return 1;
    return 3. * (sin(p * r) / (p * p * p * r * r * r) - cos(p * r) / (p * p * r * r));
  }
  if (which == 1) return exp(-p * p * r * r / 2.);
  if (which == 2) {
    if (p > (ntable - 1) * dp) return table[ntable - 1];
    return table[(int)(p / dp)];
  }
  {
    const double P = 2. * acos(-1.) / r;
    return p < P ? 1 : 0;
  }
}

/* |p| of a stored mode (px, py <= N/2, pz) as apply_filter computes it
 * (filter.cpp:76-99). */
static double flt_pabs(int px, int py, int pz, int N, double a) {
  double nu, ppx, ppy;
  if (pz == 0) nu = 0;
  else if (pz < N / 2 + 1) nu = 2.0 / (a) * sin((pz) * acos(-1.) / N);
  else nu = -2.0 / (a) * sin((pz) * acos(-1.) / N);
  if (px < N / 2 + 1) ppx = 2.0 / (a) * sin(px * acos(-1.) / N);
  else ppx = -2.0 / (a) * sin(px * acos(-1.) / N);
  ppy = 2.0 / (a) * sin(py * acos(-1.) / N);
  return sqrt(sqr(ppx) + sqr(ppy) + sqr(nu));
}

/* apply_filter(r_filter, which) (filter.cpp:53-133), one rank: each
 * component of Phi and Pi goes to momentum space (fftXtoP_direct, x a^3),
 * every mode is multiplied by W(r, |p|) -- a mode with py > N/2, which the
 * reference holds as its conjugate, takes the conjugate's |p| -- and back
 * (fftPtoX_direct, / L^3) into the interior.  which: 0 top hat, 1 Gaussian,
 * 2 tabulated (table[ntable], spacing dp), 3 sharp cut at 2 pi / r. */
int orc_apply_filter(const orc_params *p, double *Phi, double *Pi, double r, int which, const double *table,
                     int ntable, double dp) {
  const int N = p->N, Nc = p->Nc;
  const long NN = (long)N * N, V = NN * N;
  double *re = (double *)malloc(sizeof(double) * V), *im = (double *)malloc(sizeof(double) * V);
  double *wr = (double *)malloc(sizeof(double) * N), *wi = (double *)malloc(sizeof(double) * N);
  const double Norm = sqr(p->a * N) * N * p->a;
  for (int f = 0; f < 2; f++)
    for (int c = 0; c < Nc; c++) {
      double *fld = f == 0 ? Phi : Pi;
      forward_fft(p, fld, c, re, im); /* re/im[kx + N ky + N^2 kz], x a^3 */
      for (int kz = 0; kz < N; kz++)
        for (int ky = 0; ky < N; ky++)
          for (int kx = 0; kx < N; kx++) {
            int px = kx, py = ky, pz = kz;
            if (ky > N / 2) { px = mod(N - kx, N); py = N - ky; pz = mod(N - kz, N); }
            const double w = flt_w(which, r, flt_pabs(px, py, pz, N, p->a), table, ntable, dp);
            const long i = kx + (long)N * ky + NN * kz;
            re[i] *= w;
            im[i] = -(im[i] * w); /* conjugate in: the inverse is conj(DFT(conj)) */
          }
      for (long q = 0; q < NN; q++) dft_line(re + q * N, im + q * N, N, 1, wr, wi);
      for (int z = 0; z < N; z++)
        for (int x = 0; x < N; x++) dft_line(re + x + NN * z, im + x + NN * z, N, N, wr, wi);
      for (long q = 0; q < NN; q++) dft_line(re + q, im + q, N, NN, wr, wi);
      for (int z = 0; z < N; z++)
        for (int y = 0; y < N; y++)
          for (int x = 0; x < N; x++) fld[c + pos3(p, x, y, z + 1)] = re[x + N * y + NN * z] / Norm;
    }
  free(re); free(im); free(wr); free(wi);
  return 0;
}

/* Print_fp (momentumspace.cpp:280-384) per-bin columns, for bins with a
 * non-zero count and F: p, count, omega, F/(L^3 count), K/(L^3 count),
 * sqrt(FK)/(L^3 count), F p^3 /(2 pi^2 L^3 count).  cols[k*7 + ...]; rows of
 * skipped bins are zero with count 0.  Components are averaged as :471-474. */
void orc_spectrum_columns(const orc_params *p, const double *F, const double *K, const double *Q,
                          const int *counts, int nb, double *cols) {
  const int N = p->N, Nc = p->Nc;
  double binsize;
  int nbb;
  orc_spectrum_bins(p, &nbb, &binsize);
  double NormCorr = 1. / (sqr(N * p->a) * N * p->a);
  for (int k = 0; k < nb; k++) {
    double *c = cols + (long)k * 7;
    for (int j = 0; j < 7; j++) c[j] = 0.0;
    double norm2 = (counts[k] == 0 ? 0 : 1 / (double)(counts[k]));
    double pabs = binsize * k;
    if (norm2 != 0 && F[k * Nc] != 0) {
      double FF = 0, KK = 0, QQ = 0;
      for (int a = 0; a < Nc; a++) { FF += F[k * Nc + a]; KK += K[k * Nc + a]; QQ += Q[k * Nc + a]; }
      FF /= Nc; KK /= Nc; QQ /= Nc;
      (void)QQ;
      c[0] = pabs;
      c[1] = counts[k];
      c[2] = sqrt(KK / FF);
      c[3] = FF * NormCorr * norm2;
      c[4] = KK * NormCorr * norm2;
      c[5] = sqrt(FF * KK) * NormCorr * norm2;
      c[6] = FF * NormCorr * norm2 * pabs * pabs * pabs / 2. / acos(-1.) / acos(-1.);
    }
  }
}

/* ------------------------------------------------------------------ islands */
/* Per-site energy density, the summand of the reference's Energy
 * (fieldanalysis.cpp:437-471,571-579): 1/2 sum_a pi_a^2 + 1/2 sum_a grad_a
 * + V, plus the expanding box's sum_a (phi_a^2 (H0/sf)^2 / 2 - phi_a pi_a
 * H0/sf) (:626-629).  Its lattice mean is the reference's Energy. */
double orc_site_energy_at(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi, long Kooo0,
                          int x, int y, int z) {
  const int N = p->N, Nc = p->Nc;
  const double sf = clock_sf(p, c);
  long Kooo = Kooo0;
  long Kuoo = pos3(p, mod(x + 1, N), y, z), Kouo = pos3(p, x, mod(y + 1, N), z), Koou = pos3(p, x, y, z + 1);
  double kin = 0., grad = 0., inter = 0., locPhiSqr = 0., locPhi = 0., phi2 = 0., phipi = 0.;
  for (int a = 0; a < Nc; a++) {
    kin += sqr(Pi[Kooo]);
    locPhiSqr += sqr(Phi[Kooo]);
    locPhi += Phi[Kooo];
    phi2 += sqr(Phi[Kooo]);
    phipi += Phi[Kooo] * Pi[Kooo];
    grad += (sqr(Phi[Kuoo] - Phi[Kooo]) / sqr(p->a) + sqr(Phi[Kouo] - Phi[Kooo]) / sqr(p->a) +
             sqr(Phi[Koou] - Phi[Kooo]) / sqr(p->a));
    inter += component_interaction(p, Phi[Kooo], a, sf);
    Kooo++; Kuoo++; Kouo++; Koou++;
  }
  inter += site_interaction(p, locPhiSqr, locPhi, sf);
  double e = 0.5 * kin + 0.5 * grad + inter;
  if (p->expansion) e += (0.5 * phi2 * sqr(p->H0 / sf) - phipi * p->H0 / sf);
  return e;
}

double orc_site_energy(const orc_params *p, const double *Phi, const double *Pi, long K, int x, int y, int z) {
  return orc_site_energy_at(p, NULL, Phi, Pi, K, x, y, z);
}

/* Mask: mode 0 is is_island() (islands.cpp:76): the first component at the
 * site satisfies Phi^2/2 + Pi^2/2 > thres^2/2; mode 1 is the energy-density
 * mask rho(x) > thres. */
/* Delta, the per-site energy density of CalculateVolumeAverages with
 * withEnergyPS 1 (fieldanalysis.cpp:446-560): for every component of every
 * interior site, 0.5 Pi^2 plus the full squared forward differences (no 1/2)
 * plus the potential in Delta's own forms, static or expanding box.  out[]
 * holds the reference layout's interior (Nc N^3 values, index K - N^2 Nc).
 * The reference compiles these forms for theories 2-5 only (its theory 0 and
 * 1 forms name the monodromy mass, which only theory 3 defines): -1 for 0, 1. */
int orc_delta_at(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi, double *out) {
  if (p->theory < 2) return -1;
  const int N = p->N, Nc = p->Nc;
  const double mass = p->m_sqr, a2 = sqr(p->a);
  const double sf = p->expansion ? clock_sf(p, c) : 1.0;
  const long off = pos3(p, 0, 0, 1);
  for (int z = 1; z < N + 1; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) {
        const long K0 = pos3(p, x, y, z), Ku = pos3(p, mod(x + 1, N), y, z), Kv = pos3(p, x, mod(y + 1, N), z),
                   Kw = pos3(p, x, y, z + 1);
        for (int a = 0; a < Nc; a++) {
          const long K = K0 + a;
          const double ph = Phi[K];
          double d = (0.5 * sqr(Pi[K]) + sqr(Phi[Ku + a] - ph) / a2 + sqr(Phi[Kv + a] - ph) / a2 +
                      sqr(Phi[Kw + a] - ph) / a2);
          if (p->expansion) {
            d += (0.5 * sqr(p->H0 / sf) * sqr(ph) - ph * Pi[K] * p->H0 / sf);
            switch (p->theory) { /* fieldanalysis.cpp:536-558 */
              case 2:
                d += sqr(sf * sf * mass) * (1. - cos(ph / (sf * sqrt(mass))));
                break;
              case 3:
                d += (0.5 * p->m_mono_sqr * (sqr(sf)) * sqr(ph));
                d += sqr(sf * sf * mass) * (1. - cos(ph / (sf * sqrt(mass))));
                break;
              case 4:
                d += (double)(p->mass_mode) * 0.5 * mass * sf * sf * sqr(ph);
                d += (((-p->g * sf * sqr(ph) * ph) / (6.0)) + (double)(p->lambda_mode) * (sqr(sqr(ph)) / (24.0 * Nc)));
                break;
              default:
                d += sqr(sf * sf * mass) * 0.5 / p->p_mono * (pow((1. + ph * ph / mass / sf / sf), p->p_mono) - 1.);
            }
          } else {
            switch (p->theory) { /* fieldanalysis.cpp:511-535 */
              case 2:
                d += sqr(mass) * (1. - cos(ph / (sqrt(mass))));
                break;
              case 3:
                d += 0.5 * p->m_mono_sqr * sqr(ph);
                d += sqr(mass) * (1. - cos(ph / (sqrt(mass))));
                break;
              case 4:
                d += (double)(p->mass_mode) * 0.5 * mass * sqr(ph);
                d += (((-p->g * sqr(ph) * ph) / (6.0)) + (double)(p->lambda_mode) * (sqr(sqr(ph)) / (24.0 * Nc)));
                break;
              default:
                d += sqr(mass) * 0.5 / p->p_mono * (pow((1. + ph * ph / mass), p->p_mono) - 1.);
            }
          }
          out[K - off] = d;
        }
      }
  return 0;
}

int orc_delta(const orc_params *p, const double *Phi, const double *Pi, double *out) {
  return orc_delta_at(p, NULL, Phi, Pi, out);
}

static unsigned char *make_mask(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi,
                                double thres, int mode, const double *delta) {
  const int N = p->N;
  const long n = field_len(p);
  unsigned char *m = (unsigned char *)calloc((size_t)n, 1);
  for (int z = 1; z < N + 1; z++)
    for (int y = 0; y < N; y++)
      for (int x = 0; x < N; x++) {
        long K = pos3(p, x, y, z);
        if (mode == 0)
          m[K] = (Phi[K] * Phi[K] * 0.5 + Pi[K] * Pi[K] * 0.5 > thres * thres * 0.5);
        else if (mode == 2) /* EnergybasedID: Delta[K] > thres (islands.cpp:82-83) */
          m[K] = delta[K - pos3(p, 0, 0, 1)] > thres;
        else
          m[K] = orc_site_energy_at(p, c, Phi, Pi, K, x, y, z) > thres;
      }
  return m;
}

/* The expanding box's island energy terms (islands.cpp:136-196): the
 * kinetic term with its H0/sf parts, and the potential added in the
 * reference's separate steps. */
static void bfs_expanded(const orc_params *p, double phi, double pi, double sf, double *cKinEn, double *cPotEn) {
  const int Nc = p->Nc;
  const double mass = p->m_sqr, H0 = p->H0;
  *cKinEn += (0.5 * sqr(pi) + 0.5 * sqr(H0 / sf) * sqr(phi) - phi * pi * H0 / sf);
  switch (p->theory) {
    case 0:
      *cPotEn += (double)(p->mass_mode) * 0.5 * mass * sf * sf * sqr(phi);
      *cPotEn += (double)(p->lambda_mode) * (sqr(sqr(phi)) / (24.0 * Nc)) +
                 (sqr(sqr(phi)) * sqr(phi) / (720.0 * Nc * Nc * p->kappa * p->kappa * sf * sf));
      break;
    case 1:
      *cPotEn += (double)(p->mass_mode) * 0.5 * mass * sf * sf * sqr(phi);
      *cPotEn += (p->h * phi * sf * sf * sf + (double)(p->lambda_mode) * (sqr(sqr(phi)) / (24.0 * Nc)));
      break;
    case 2:
      *cPotEn += sqr(sf * sf * mass) * (1. - cos(phi / (sf * sqrt(mass))));
      break;
    case 3:
      *cPotEn += (0.5 * p->m_mono_sqr * (sqr(sf)) * sqr(phi));
      *cPotEn += sqr(sf * sf * mass) * (1. - cos(phi / (sf * sqrt(mass))));
      break;
    case 4:
      *cPotEn += (double)(p->mass_mode) * 0.5 * mass * sf * sf * sqr(phi);
      *cPotEn += (((-p->g * sf * sqr(phi) * phi) / (6.0)) + (double)(p->lambda_mode) * (sqr(sqr(phi)) / (24.0 * Nc)));
      break;
    default:
      *cPotEn += sqr(sf * sf * mass) * 0.5 / p->p_mono * (pow((1. + phi * phi / mass / sf / sf), p->p_mono) - 1.);
  }
}

/* One BFS (islands.cpp:90-279) from seed P with label `flag`; sf > 0 selects
 * the expanding box's energies.  z is open (1..N) as on one rank (:224-236)
 * unless zper. */
static void bfs(const orc_params *p, const double *Phi, const double *Pi, const unsigned char *mask, int *b,
                long *queue, long P, int flag, int zper, orc_island *B, double sf, const double *delta) {
  const long doff = pos3(p, 0, 0, 1);
  const int N = p->N, Nc = p->Nc;
  const double mass = p->m_sqr;
  int NN = 0;
  double cPotEn = 0., cGradEn = 0., cKinEn = 0., cavPhi = 0.;
  long cnt = P;
  long head = 0, tail = 0;
  b[P] = flag;
  queue[tail++] = P;
  while (head < tail) {
    long Kooo = queue[head++];
    if (delta) { /* EnergybasedID: the peak of Delta (islands.cpp:113-114) */
      if (delta[Kooo - doff] > delta[cnt - doff]) cnt = Kooo;
    } else if (Phi[Kooo] * Phi[Kooo] > Phi[cnt] * Phi[cnt]) {
      cnt = Kooo;
    }
    int z = (int)(Kooo / ((long)Nc * N * N));
    int y = (int)((Kooo - (long)Nc * N * N * z) / ((long)Nc * N));
    int x = (int)((Kooo - (long)Nc * N * N * z - (long)Nc * N * y) / Nc);
    long Kuoo = pos3(p, mod(x + 1, N), y, z);
    long Kdoo = pos3(p, mod(x - 1, N), y, z);
    long Kouo = pos3(p, x, mod(y + 1, N), z);
    long Kodo = pos3(p, x, mod(y - 1, N), z);
    long Koou = pos3(p, x, y, z + 1);
    long Kood = pos3(p, x, y, z - 1);
    NN++;
    cGradEn += 0.5 * (sqr(Phi[Kuoo] - Phi[Kooo]) + sqr(Phi[Kouo] - Phi[Kooo]) + sqr(Phi[Koou] - Phi[Kooo])) / sqr(p->a);
    if (sf > 0)
      bfs_expanded(p, Phi[Kooo], Pi[Kooo], sf, &cKinEn, &cPotEn);
    else
      cKinEn += 0.5 * sqr(Pi[Kooo]);
    if (sf > 0)
      ; /* potential added by bfs_expanded */
    else if (p->theory == 0)
      cPotEn += (double)(p->mass_mode) * 0.5 * mass * sqr(Phi[Kooo]) +
                (double)(p->lambda_mode) * (sqr(sqr(Phi[Kooo])) / (24.0 * Nc)) +
                (sqr(sqr(Phi[Kooo])) * sqr(Phi[Kooo]) / (720.0 * Nc * Nc * p->kappa * p->kappa));
    else if (p->theory == 1)
      cPotEn += (p->h * Phi[Kooo] + (double)(p->mass_mode) * 0.5 * mass * sqr(Phi[Kooo]) +
                 (double)(p->lambda_mode) * (sqr(sqr(Phi[Kooo])) / (24.0 * Nc)));
    else if (p->theory == 2) /* islands.cpp:160-167 */
      cPotEn += sqr(mass) * (1. - cos(sqrt(sqr(Phi[Kooo]) / mass)));
    else if (p->theory == 3) /* :169-177 */
      cPotEn += 0.5 * p->m_mono_sqr * sqr(Phi[Kooo]) + sqr(mass) * (1. - cos(sqrt(sqr(Phi[Kooo]) / mass)));
    else if (p->theory == 4) /* :179-187 */
      cPotEn += (double)(p->mass_mode) * 0.5 * mass * sqr(Phi[Kooo]) - p->g * sqr(Phi[Kooo]) * Phi[Kooo] / 6. +
                (double)(p->lambda_mode) * (sqr(sqr(Phi[Kooo])) / (24.0 * Nc));
    else /* :189-196 */
      cPotEn += sqr(mass) * 0.5 / p->p_mono * (pow((1. + Phi[Kooo] * Phi[Kooo] / mass), p->p_mono) - 1.);
    cavPhi += Phi[Kooo];
    if (mask[Kuoo] && b[Kuoo] == -1) { b[Kuoo] = flag; queue[tail++] = Kuoo; }
    if (mask[Kdoo] && b[Kdoo] == -1) { b[Kdoo] = flag; queue[tail++] = Kdoo; }
    if (mask[Kouo] && b[Kouo] == -1) { b[Kouo] = flag; queue[tail++] = Kouo; }
    if (mask[Kodo] && b[Kodo] == -1) { b[Kodo] = flag; queue[tail++] = Kodo; }
    if (zper) {
      long Kp = pos3(p, x, y, z == N ? 1 : z + 1), Km = pos3(p, x, y, z == 1 ? N : z - 1);
      if (mask[Kp] && b[Kp] == -1) { b[Kp] = flag; queue[tail++] = Kp; }
      if (mask[Km] && b[Km] == -1) { b[Km] = flag; queue[tail++] = Km; }
    } else {
      if (z < N)
        if (mask[Koou] && b[Koou] == -1) { b[Koou] = flag; queue[tail++] = Koou; }
      if (z > 1)
        if (mask[Kood] && b[Kood] == -1) { b[Kood] = flag; queue[tail++] = Kood; }
    }
  }
  cavPhi /= (double)(NN);
  const double cell = p->a * p->a * p->a;
  B->index = flag;
  B->size = NN;
  B->volume = NN * p->a * p->a * p->a;
  B->pot_en = cPotEn * cell;
  B->kin_en = cKinEn * cell;
  B->grad_en = cGradEn * cell;
  B->av_phi = cavPhi;
  B->peak_pos = (double)cnt;
  B->peak_value = delta ? delta[cnt - doff] : Phi[cnt]; /* islands.cpp:256-261 */
  B->seed_pos = (double)P;
}

/* Full_Analysis() from an empty island history (islands.cpp:778-840): labels
 * reset to -1, then every unlabelled mask site in linear order seeds a BFS.
 * Island i gets label i, so labels follow each island's smallest site index.
 * labels (may be NULL) uses the reference layout; islands[] receives at most
 * max_islands records.  Returns the island count, or -1 on allocation failure. */
int orc_islands_at(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi, double thres,
                   int mode, int zper, int *labels, orc_island *islands, int max_islands) {
  const int N = p->N, Nc = p->Nc;
  const long n = field_len(p);
  const double sf = p->expansion ? clock_sf(p, c) : 0.0;
  double *delta = NULL;
  if (mode == 2) {
    delta = (double *)malloc(sizeof(double) * (size_t)Nc * N * N * N);
    if (!delta) return -1;
    if (orc_delta_at(p, c, Phi, Pi, delta)) {
      free(delta);
      return -2;
    }
  }
  unsigned char *mask = make_mask(p, c, Phi, Pi, thres, mode, delta);
  int *b = labels ? labels : (int *)malloc(sizeof(int) * (size_t)n);
  long *queue = (long *)malloc(sizeof(long) * (size_t)n);
  if (!mask || !b || !queue) return -1;
  for (long k = 0; k < n; k++) b[k] = -1;
  int count = 0;
  orc_island scratch;
  for (long K = pos3(p, 0, 0, 1); K < (long)Nc * N * N * (N + 1); K++)
    if (mask[K] && b[K] == -1) {
      orc_island *B = count < max_islands ? &islands[count] : &scratch;
      bfs(p, Phi, Pi, mask, b, queue, K, count, zper, B, sf, delta);
      count++;
    }
  free(mask);
  free(queue);
  free(delta);
  if (!labels) free(b);
  return count;
}

/* The density-contrast spectrum of Calculate_CorrelationFunctions with
 * withEnergyPS 1 (momentumspace.cpp:165-183, 191, 233-270): Delta, its mean
 * Aavden = (sum over every component of every site) / N^3, the contrast
 * (Delta - Aavden) / Aavden per component, and its binned power
 * D[bin*Nc + a] with orc_spectrum's modes, weights and a^3 factors (the
 * reference transforms Delta with the same fftXtoP_direct as Phi).  Returns
 * the bin count as orc_spectrum does, -2 for the theories without Delta. */
int orc_spectrum_energy_at(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi, double *D,
                           int *counts) {
  const int N = p->N, Nc = p->Nc;
  const long nint = (long)Nc * N * N * N, off = pos3(p, 0, 0, 1);
  double *delta = (double *)malloc(sizeof(double) * (size_t)nint);
  double *field = (double *)calloc((size_t)field_len(p), sizeof(double));
  if (!delta || !field) {
    free(delta);
    free(field);
    return -1;
  }
  if (orc_delta_at(p, c, Phi, Pi, delta)) {
    free(delta);
    free(field);
    return -2;
  }
  double aavden = 0.;
  for (long k = 0; k < nint; k++) aavden += delta[k];
  const double Aavden = aavden / ((double)N * N * N);
  for (long k = 0; k < nint; k++) {
    double v = delta[k];
    v -= Aavden;
    v /= Aavden;
    field[off + k] = v;
  }
  int nb;
  double binsize;
  orc_spectrum_bins(p, &nb, &binsize);
  double *K = (double *)malloc(sizeof(double) * (size_t)nb * Nc), *Q = (double *)malloc(sizeof(double) * (size_t)nb * Nc);
  const int r = (K && Q) ? orc_spectrum(p, field, field, D, K, Q, counts) : -1;
  free(K);
  free(Q);
  free(delta);
  free(field);
  return r;
}

int orc_islands(const orc_params *p, const double *Phi, const double *Pi, double thres, int mode, int zper,
                int *labels, orc_island *islands, int max_islands) {
  return orc_islands_at(p, NULL, Phi, Pi, thres, mode, zper, labels, islands, max_islands);
}

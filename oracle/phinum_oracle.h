/*
 * phinum_oracle.h -- CPU restatement of PhiNum's lattice hot path.
 * TEST INFRASTRUCTURE: see phinum_oracle.c.
 */
#ifndef PHINUM_ORACLE_H
#define PHINUM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_NC 4

/* Run parameters, in the reference's own terms (parameters.cpp:84-201). */
typedef struct orc_params {
  int N;           /* N_t = N_eta: cubic lattice edge */
  int Nc;          /* field components */
  int theory;      /* 0: phi^4 + phi^6 (Kappa), 1: phi^4 + linear h, 2-5 (parameters.cpp:122-170) */
  int mass_mode;   /* Mass_Mode */
  int lambda_mode; /* Lambda_Mode */
  int expansion;   /* 0 static box, 1 expanding box (radiation era, H_0) */
  double a;        /* a_t = a_eta */
  double dt;       /* dtBaseTrans: dtau = dt * a */
  double T0;
  double m_sqr;    /* M_sqr (= BareM_sqr_long/_trans without tadpole renormalisation) */
  double kappa;    /* Kappa (theory 0) */
  double h;        /* h (theory 1) */
  double g;        /* g (theory 4) */
  double p_mono;   /* p_mono (theory 5) */
  double m_mono_sqr; /* M_mono_sqr (theory 3) */
  double H0;       /* H_0 (expansion 1, parameters.cpp:177) */
} orc_params;

/* numeric:: and LocalLattice:: time keeping (dynamics.cpp:8-50). */
typedef struct orc_clock {
  double tau, dtau, last_mom, last_field;
  int steps, pad_;
  /* expanding box (dynamics.cpp:8-50): conformal time, scale factor and the
   * conformal update stamps; tau and 1 for the static box */
  double tau_c, sf, last_mom_c, last_field_c;
} orc_clock;

/* One SO row: CalculateVolumeAverages + CalculateExtrema outputs
 * (lattice.cpp:44-58).  Positions are indices into the reference layout. */
typedef struct orc_row {
  double t;
  double phi[ORC_MAX_NC], pi[ORC_MAX_NC];
  double phi2, pi2, phipi, phi4, phi6;
  double energy, interaction, charge;
  double min_phi, max_phi, max_abs_phi;
  double min_pos, max_pos, max_abs_pos;
  double gradient; /* GradPhiSqr / vol: mean of sum_d (forward difference)^2 / a^2 */
  double reserved[2];
} orc_row;

/* One island (struct island, islands.cpp:13-28, latest entries). */
typedef struct orc_island {
  double index, size, volume, pot_en, kin_en, grad_en, av_phi, peak_pos, peak_value, seed_pos;
} orc_island;

/* Parameters of SetInitialConditions for `initialize 3` (the reference's
 * globals of the same names, parameters.cpp; M2_long/M2_trans as
 * renormalization.cpp:17-18 sets them). */
typedef struct orc_ic {
  long seed;  /* srand48 argument */
  int justnoise, pad_;
  double QS, scale2, amplitude, noise;
  double phi0[2], pi0[2];
  double m2_long, m2_trans;
  /* the `initialize` (0-4) and `withcharge` switches and the globals of
   * initialize 0-2 (parameters.cpp:207-272): chi, FAmp, Lambda,
   * Temperature and the homogeneous phi0, pi0 of component 0 */
  int initialize, withcharge;
  double chi, famp, lambda, temperature, phi0s, pi0s;
} orc_ic;

int orc_version(void);
int orc_max_threads(void);
void orc_reset(const orc_params *p, orc_clock *c);
void orc_exchange(const orc_params *p, double *f);
void orc_evolve(const orc_params *p, orc_clock *c, double *Phi, double *Pi, int nsteps, int nthreads);

/* The reference's single-precision build (doubleprecision -1: pseudo_double
 * = float, parameters.cpp:13-16): clock and fields in float, theories 0 and
 * 1, static box. */
typedef struct orc_clock_f32 {
  float tau, dtau, last_mom, last_field;
  int steps, pad_;
} orc_clock_f32;
void orc_reset_f32(const orc_params *p, orc_clock_f32 *c);
void orc_evolve_f32(const orc_params *p, orc_clock_f32 *c, float *Phi, float *Pi, int nsteps, int nthreads);
void orc_averages(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi, orc_row *o);
int orc_run_loop(const orc_params *p, orc_clock *c, double *Phi, double *Pi, int nsteps, double tso,
                 orc_row *rows, int max_rows, int nthreads);
void orc_spectrum_bins(const orc_params *p, int *nbins, double *binsize);
int orc_initial_conditions(const orc_params *p, const orc_ic *ic, double *Phi, double *Pi);
int orc_apply_filter(const orc_params *p, double *Phi, double *Pi, double r, int which, const double *table,
                     int ntable, double dp);
int orc_spectrum(const orc_params *p, const double *Phi, const double *Pi, double *F, double *K, double *Q,
                 int *counts);
int orc_spectrum_uniform(const orc_params *p, const double *Phi, const double *Pi, int nbins, double *F, double *K,
                         double *Q, int *counts);
void orc_spectrum_columns(const orc_params *p, const double *F, const double *K, const double *Q,
                          const int *counts, int nb, double *cols);
double orc_site_energy(const orc_params *p, const double *Phi, const double *Pi, long K, int x, int y, int z);
int orc_islands_at(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi, double thres,
                   int mode, int zper, int *labels, orc_island *islands, int max_islands);
double orc_site_energy_at(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi, long K,
                          int x, int y, int z);
int orc_islands(const orc_params *p, const double *Phi, const double *Pi, double thres, int mode, int zper,
                int *labels, orc_island *islands, int max_islands);
/* withEnergyPS 1: Delta per component (interior, Nc N^3), the island mask
 * mode 2 (Delta > thres, peak and Peak_value by Delta) and the contrast
 * spectrum; theories 2-5 as the reference compiles them. */
int orc_delta_at(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi, double *out);
int orc_delta(const orc_params *p, const double *Phi, const double *Pi, double *out);
int orc_spectrum_energy_at(const orc_params *p, const orc_clock *c, const double *Phi, const double *Pi, double *D,
                           int *counts);

#ifdef __cplusplus
}
#endif
#endif

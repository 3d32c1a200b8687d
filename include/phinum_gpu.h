/*
 * phinum_gpu.h -- C ABI of the GB300 (sm_103a) implementation of PhiNum's
 * lattice hot path: leapfrog evolution of (phi, pi) on a periodic cubic
 * lattice with fused volume averages, the radial power spectrum after an R2C
 * FFT, and island (connected-component) labelling.
 *
 * The reference exposes no FFI: its entry points are argument-less free
 * functions over globals.  Each call below replaces one of them; the host
 * keeps the reference's parameters and lattice layout and copies results
 * into the same globals (see phinum_gb300/adapter/phinum_dynamics.cpp).
 *
 * Conventions
 *   - Every function returns an int status: PHN_OK (0) or a negative
 *     PHN_ERR_* code.  Nothing aborts or traps; phn_last_error() gives text.
 *   - Host field arrays use the reference layout (lattice.cpp:76-78,
 *     util.cpp:34-37): Nc*N*N*(N+2) doubles, index Nc*(x + N*y + N*N*z) + a,
 *     z-slabs 0 and N+1 are ghost copies of slabs N and 1.  The caller owns
 *     them; the handle owns its device copies.
 *   - Positions reported (extrema, island peaks) are indices into that layout.
 *   - One handle = one lattice on the current CUDA device, one stream.
 *     Calls on a handle are not thread-safe; distinct handles are independent.
 */
#ifndef PHINUM_GPU_H
#define PHINUM_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PHN_ABI_VERSION 4
#define PHN_MAX_NC 4

enum {
  PHN_OK = 0,
  PHN_ERR_INVALID = -1,     /* bad argument or parameter */
  PHN_ERR_CUDA = -2,        /* a CUDA runtime or cuFFT call failed */
  PHN_ERR_NONFINITE = -3,   /* a reduction saw NaN or Inf in the fields */
  PHN_ERR_TIMEOUT = -4,     /* a bounded device-side wait gave up */
  PHN_ERR_NOMEM = -5,       /* device allocation failed or exceeds the size cap */
  PHN_ERR_UNSUPPORTED = -6, /* valid in the reference, not provided here */
  PHN_ERR_TRUNCATED = -7    /* output buffer smaller than the result */
};

enum {
  PHN_FP64 = 0,      /* fields and arithmetic in FP64, in the reference's operation order */
  PHN_FP32 = 1,      /* fields in FP32, FP64 reductions */
  PHN_FP32_KAHAN = 2, /* fields in FP32 with compensated (Kahan) kick and drift, FP64 reductions */
  PHN_FP32_PAIR = 3   /* FP32 pairs: double-float arithmetic on the FP32 pipe (about 48 bits);
                         the adjoint's forward solve only (phn_adjoint_set_forward_precision) */
};

enum {
  PHN_ISLAND_REFERENCE = 0, /* is_island(): phi^2/2 + pi^2/2 > thres^2/2 (islands.cpp:76) */
  PHN_ISLAND_ENERGY = 1,    /* energy density rho(x) > thres, rho the summand of <E> */
  PHN_ISLAND_DELTA = 2      /* EnergybasedID 1 (islands.cpp:82-83): Delta(x) > thres, Delta the per-site
                               energy density of withEnergyPS 1 (fieldanalysis.cpp:446-560: 0.5 Pi^2, the
                               full squared forward differences, the potential); the peak and its value by
                               Delta (islands.cpp:113-114, 259-260).  Theories 2-5, as the reference compiles
                               it; the reference's Full_Analysis takes thres = 4 <rho> (islands.cpp:783-786) */
};

/* Run parameters, in the reference's own terms (parameters.cpp:84-201). */
typedef struct phn_params {
  int N;           /* N_t = N_eta: lattice edge (cubic box) */
  int Nc;          /* field components, 1..PHN_MAX_NC */
  int potential;   /* the reference's `theory` (parameters.cpp:86-170): 0 phi^4 + phi^6 (Kappa),
                      1 phi^4 + linear h, 2 cosine, 3 cosine + monodromy mass,
                      4 cubic (g), 5 power-law monodromy (p_mono); every theory for Nc 1-4.
                      Named apart because the reference #defines `theory` in the
                      translation unit that includes this */
  int mass_mode;   /* Mass_Mode */
  int lambda_mode; /* Lambda_Mode */
  int precision;   /* PHN_FP64 / PHN_FP32 / PHN_FP32_KAHAN */
  double a;        /* a_t = a_eta */
  double dt;       /* dtBaseTrans; dtau = dt * a (dynamics.cpp:42) */
  double T0;       /* initial time */
  double m_sqr;    /* M_sqr (bare masses without tadpole renormalisation) */
  double kappa;    /* Kappa, theory 0 */
  double h;        /* h, theory 1 */
  double g;        /* g, theory 4 */
  double p_mono;   /* p_mono, theory 5 */
  double m_mono_sqr; /* M_mono_sqr, theory 3 */
  int expanding;   /* the reference's `expansion` switch: 0 static box, 1 radiation-era
                      expanding box, a = sqrt(1 + 2 H_0 tau), kick and drift in conformal
                      time (dynamics.cpp:36-50, :88-163, :185-212).  Named apart because
                      the reference #defines `expansion` */
  int reserved_;   /* zero */
  double H0;       /* H_0 (parameters.cpp:177), expansion 1 */
} phn_params;

/* One SO row: the outputs of CalculateVolumeAverages + CalculateExtrema
 * (lattice.cpp:44-58), as 26 doubles. */
typedef struct phn_averages {
  double t;                               /* time stamp (SO rows: LastSOoutput) */
  double phi[PHN_MAX_NC], pi[PHN_MAX_NC]; /* avgphi[a], avgpi[a] */
  double phi2, pi2, phipi, phi4, phi6;    /* avgphi2 ... avgphi6 */
  double energy, interaction, charge;     /* avgEnergy, avgInteraction, avgCharge */
  double min_phi, max_phi, max_abs_phi;   /* GlminPhi, GlmaxPhi, GlmaxAbsPhi */
  double min_pos, max_pos, max_abs_pos;   /* minpos, maxpos, maxAbspos */
  double gradient;                        /* GradPhiSqr / vol */
  double nonfinite;                       /* number of non-finite phi/pi values seen */
  double scale_factor;                    /* LocalLattice::scale_factor, the expanding box's SO
                                             time column (fieldanalysis.cpp:789-791); 1 when static */
} phn_averages;

/* One island (struct island, islands.cpp:13-28).  Islands are numbered by
 * their smallest site index, which is the reference's seed order. */
typedef struct phn_island {
  double index, size, volume, pot_en, kin_en, grad_en, av_phi, peak_pos, peak_value, seed_pos;
} phn_island;

typedef struct phn_handle phn_handle;

int phn_abi_version(void);
const char *phn_last_error(void);
int phn_device_count(int *count);

/* LocalLattice::init + FFT::init + MomentumSpace::init + reset()
 * (lattice.cpp:70-104, clusterfft.cpp:36-47, momentumspace.cpp:32-65,
 * dynamics.cpp:28-50): allocates device fields (zeroed) on the current device. */
int phn_create(const phn_params *params, phn_handle **out);
/* LocalLattice::fin / FFT::fin / MomentumSpace::fin (lattice.cpp:107-117). */
int phn_destroy(phn_handle *h);

/* Replaces direct writes/reads of LocalLattice::Phi/Pi (lattice.cpp:77-78):
 * host arrays in the reference layout; upload reads the interior only.
 * download writes Phi including its ghost slabs, as Communication::exchange()
 * leaves them, and Pi's interior only: the reference never writes Pi's ghost
 * slabs, so the caller's values there are left untouched. */
int phn_upload(phn_handle *h, const double *Phi, const double *Pi);
int phn_download(phn_handle *h, double *Phi, double *Pi);
/* The same for the reference's single-precision build (doubleprecision -1,
 * pseudo_double = float; parameters.cpp:13-16): float arrays in the same
 * layout, converted on the device to the handle's precision (and back, FP64
 * handles rounding to float). */
int phn_upload_f32(phn_handle *h, const float *Phi, const float *Pi);
int phn_download_f32(phn_handle *h, float *Phi, float *Pi);

/* reset() (dynamics.cpp:28-50): tau = T0, kick/drift clocks = tau, counters 0.
 * The next evolve kicks by dtau/2 (dynamics.cpp:84). */
int phn_reset(phn_handle *h);
/* nsteps x evolve() (dynamics.cpp:196-237): updateMomenta + updateFields +
 * exchange, fused into one kernel per step. */
int phn_evolve(phn_handle *h, int nsteps);
/* LocalLattice::tau and numeric::total_stepcount. */
int phn_time(const phn_handle *h, double *tau, int *total_stepcount);
/* LocalLattice::tau_conformal and scale_factor (lattice.cpp:14-17) of the
 * expanding box; tau and 1 for the static box. */
int phn_conformal_time(const phn_handle *h, double *tau_conformal, double *scale_factor);

/* CalculateExtrema() + CalculateVolumeAverages() (fieldanalysis.cpp:319-699)
 * on the current state. */
int phn_volume_averages(phn_handle *h, phn_averages *out);
/* false_vacuum_decayed() (fieldanalysis.cpp:887-893) on the last averages. */
int phn_false_vacuum_decayed(const phn_averages *avg, int potential, int *decayed);

/* The run loop of main.cpp:685-699 with an explicit step count: reset(),
 * then nsteps x { Print_AveragesExtrema() cadence (TSO on the accumulated tau,
 * fieldanalysis.cpp:753-780); evolve() }.  The averages of a due row are
 * fused into that step's kernel (zero extra passes over HBM).  Rows are
 * stamped with LastSOoutput.  *nrows receives the number of rows; if more than
 * max_rows were due the call returns PHN_ERR_TRUNCATED after writing max_rows. */
int phn_run_loop(phn_handle *h, int nsteps, double tso, phn_averages *rows, int max_rows, int *nrows);

/* MomentumSpace::init (momentumspace.cpp:40-47): bin count and width. */
int phn_spectrum_bins(const phn_handle *h, int *nbins, double *binsize);
/* fftXtoP_direct + Calculate_CorrelationFunctions (clusterfft.cpp:185-225,
 * momentumspace.cpp:140-278) on the current state: TotalCorrF/K/Q[bin*Nc+a]
 * and TotalBCounts[bin].  Arrays hold nbins*Nc (F, K, Q) and nbins (counts). */
int phn_spectrum(phn_handle *h, double *F, double *K, double *Q, int *counts, int nbins);
/* The density-contrast spectrum of Calculate_CorrelationFunctions with
 * withEnergyPS 1 (momentumspace.cpp:165-183, 191, 233-270): Delta of every
 * component at every site (fieldanalysis.cpp:446-560), Aavden = its sum over
 * components and sites / N^3, the contrast (Delta - Aavden) / Aavden, and
 * its binned power D[bin*Nc + a] = TotalCorrD with phn_spectrum's modes,
 * weights and a^3 a^3 factor; counts as phn_spectrum's.  Theories 2-5, for
 * which the reference compiles it.  The fields are not changed (the reference
 * overwrites its Delta array with the contrast). */
int phn_spectrum_energy(phn_handle *h, double *D, int *counts, int nbins);

/* The configuration's radial spectrum (no reference counterpart): the modes,
 * weights and sums of phn_spectrum, binned uniformly in the lattice momentum
 * |p| on [0, p_max], p_max = 2 sqrt(3) / a (pTmax of momentumspace.cpp:43):
 * bin = (int)(|p| / (p_max / nbins)), the top edge in the last bin.
 * 1 <= nbins <= 1024; F, K, Q hold nbins*Nc, counts nbins. */
int phn_spectrum_uniform(phn_handle *h, int nbins, double *F, double *K, double *Q, int *counts);

/* Device time of the last phn_spectrum, phn_spectrum_uniform or
 * phn_spectrum_energy call on this handle (no reference counterpart; CUDA
 * events on the handle's stream): transform_ms, the R2C transforms of phi
 * and pi summed over the components (0 for phn_spectrum_energy, whose
 * contrast field is transformed with it); binning_ms, the binning and
 * per-bin fold kernels.  PHN_ERR_INVALID before the first spectrum call. */
int phn_spectrum_timing(const phn_handle *h, double *transform_ms, double *binning_ms);

/* SetInitialConditions() (initialconditions.cpp:45-723) for `initialize 3`,
 * static or expanding box (the handle's `expanding`, with its T0 and H0), no
 * charge, on the device: drand48's stream from srand48(seed)
 * (the reference seeds with time(NULL)*(ID+1), initialconditions.cpp:16),
 * consumed in the reference's mode order -- two phases and one polar
 * Box-Muller acceptance per mode and component -- then ensureRealResult and
 * fftPtoX (clusterfft.cpp:55-182) with cuFFT.  Writes phi and pi of the
 * handle (the clock is not reset).  The stream and its assignment to modes
 * are exact; amplitudes agree with the C library's log/sin/cos to rounding.
 * N even.  Parameters are the reference's globals of the same names. */
typedef struct phn_ic_params {
  long seed;            /* the srand48 argument */
  int justnoise;        /* justnoise */
  double QS, scale2;    /* QS, scale2 (0: no cutoff) */
  double amplitude;     /* Amplitude */
  double noise;         /* Noise */
  double phi0[2];       /* phi0_0, phi0_1 (homogeneous values of components 0, 1) */
  double pi0[2];        /* pi0_0, pi0_1 */
  double m2_long;       /* M2_long (= M_sqr without tadpole renormalisation, renormalization.cpp:17) */
  double m2_trans;      /* M2_trans (components a >= 1) */
} phn_ic_params;
int phn_initial_conditions(phn_handle *h, const phn_ic_params *ic);

/* SetInitialConditions() for the reference's other compile-time choices
 * (initialconditions.cpp:45-723; parameters.cpp:205-303): `initialize`
 *   0  parametric resonance: occupation FAmp*Lambda, Omega^2 = p^2 + |M_sqr|
 *      - 3 Temperature^2 phi0^2 / (6 Nc) (component 0; 1x for the others);
 *   1  box: occupation Amplitude below QS in sqrt(pt^2 + chi^2 pz^2), Noise
 *      below 2 QS, Omega^2 = p^2 + |M_sqr| - 3 phi0^2 / (6 Nc) (1x for a > 0);
 *   2  large-Lambda box: Amplitude + Noise below QS, Noise below scale2,
 *      Omega as initialize 1;
 *   3  phn_initial_conditions;
 *   4  Temperature / sqrt(p^2 + M2_long) + Noise below QS, Noise below
 *      scale2, Omega as initialize 3 (static forms);
 * with withcharge 1 the charged variant (:120-291): for Nc = 2 one phase and
 * one Gaussian per mode, component 0 reusing the draws of the two modes
 * before (the first mode's are the reference's uninitialized locals, taken as
 * 0); for other Nc the draws of withcharge 0, with the static forms of
 * initialize 3.  Initialize 0-2 add phi0, pi0 to component 0 only; 3 and 4
 * add phi0[], pi0[] of phn_ic_params to components 0 and 1.  phn_ic_params
 * supplies seed, justnoise, QS, scale2, Amplitude, Noise, M2_long/M2_trans
 * (and phi0[], pi0[] for 3, 4); M_sqr is the handle's.  Initialize 4 with
 * charge is PHN_ERR_UNSUPPORTED (the reference sets no occupation there). */
typedef struct phn_ic_mode {
  int init_mode;      /* the reference's `initialize` switch, 0-4 */
  int charged;        /* its `withcharge` switch, 0 or 1 (both named apart because the
                         reference #defines them in the translation unit that includes this) */
  double chi;         /* chi: anisotropy of initialize 1 */
  double famp;        /* FAmp (initialize 0) */
  double lambda;      /* Lambda (initialize 0) */
  double temperature; /* Temperature (initialize 0 and 4) */
  double phi0, pi0;   /* phi0, pi0 of initialize 0-2 */
} phn_ic_mode;
int phn_initial_conditions_mode(phn_handle *h, const phn_ic_params *ic, const phn_ic_mode *mode);

/* Full_Analysis() seeding from an empty history (islands.cpp:72-279,778-840):
 * mask (mode), 6-connectivity, x and y periodic, z open as on one rank unless
 * z_periodic.  labels (optional, reference layout, -1 outside islands) and up
 * to max_out island records; *n_islands receives the total count.  Nc must
 * be 1 (the reference's scan walks component-interleaved indices). */
int phn_islands(phn_handle *h, double thres, int mode, int z_periodic, int *labels, phn_island *out,
                int max_out, int *n_islands);

/* apply_filter(r_filter, which_filter) (filter.cpp:53-133): every component
 * of phi and pi is multiplied in momentum space by a window of |p|: a top hat
 * (W_tophat), a Gaussian (W_gaussian), a tabulated window (W_import_bounce:
 * table[min(int(|p| / dp), ntable - 1)], the reference reads it from
 * bounce.txt) or a sharp cut at 2 pi / r (W_ktophat).  Compensated FP32
 * handles restart their compensation at zero. */
enum { PHN_FILTER_TOPHAT = 0, PHN_FILTER_GAUSSIAN = 1, PHN_FILTER_TABLE = 2, PHN_FILTER_KTOPHAT = 3 };
int phn_apply_filter(phn_handle *h, double r_filter, int which, const double *table, int ntable, double dp);

/* SaveConfig(Name) (fieldanalysis.cpp:252-283): writes <dir>/field-<name>-<rank>.out,
 * one line "%.17e %.17e\n" of Phi and Pi per interior site in the reference
 * layout's order ("%.9e %.9e\n" of the float values for PHN_FP32 handles, as
 * the reference's single-precision build writes), and for rank 0
 * <dir>/moment-<name>.out with tau as an ostream prints it.  The bytes are the
 * reference's; lines are formatted on nthreads host threads (0: all cores).
 * dir NULL or "" means the working directory, as the reference uses. */
int phn_save_config(phn_handle *h, const char *dir, int name, int rank, int nthreads);
/* ExtractConfig(Name) (fieldanalysis.cpp:285-312): reads those files into the
 * handle; *t0 (optional) receives the time stamp, which the reference
 * assigns to T0. */
int phn_load_config(phn_handle *h, const char *dir, int name, int rank, double *t0, int nthreads);
/* The file formatting and parsing alone, on host arrays in the reference
 * layout (interior slabs; no device involved). */
int phn_write_config_file(const char *path, const double *Phi, const double *Pi, int N, int Nc, int precision,
                          int nthreads);
int phn_read_config_file(const char *path, double *Phi, double *Pi, int N, int Nc, int nthreads);

/* phn_islands without the host copies: every island's record is assembled
 * in a device buffer held by the handle, *d_records points at it (NULL when
 * there is no island) and *n_islands receives the count.  The records stay
 * valid until the next island call on the handle or its destruction; the
 * labels stay on the device for phn_islands_lookup.  The same records as
 * phn_islands writes, for callers that consume them on the GPU. */
int phn_islands_device(phn_handle *h, double thres, int mode, int z_periodic, const phn_island **d_records,
                       int *n_islands);

/* After phn_islands: the island (numbered as phn_islands numbers them) that
 * holds each queried site, reference-layout indices; -1 outside the mask. */
int phn_islands_lookup(phn_handle *h, const long long *pos, int n, int *island);

/* ---- Island tracking over a run -------------------------------------------
 * Full_Analysis() with its history (islands.cpp:651-840): island_analysis::
 * found_islands is held by a tracker.  Each update sorts the tracked islands
 * by their last volume (std::sort with the reference's ordering), retires
 * those whose centre left the mask (Old_islands), re-seeds the others from
 * their centres in that order -- an island whose centre lies in an island
 * already claimed this update is merged away -- appends one history entry
 * (at most 5 kept: the first two and the last three, islands.cpp:264-276),
 * sets status 1 for an expanding bubble (is_bubble, reported once per
 * update as print_bubble_history does) or 2 for an oscillon (is_oscillon),
 * and adds the unclaimed islands as new ones in the reference's scan order,
 * numbered number_of_islands + rank * 1000000. */
#define PHN_TRACK_HISTORY 5
typedef struct phn_track_island {
  double index, status, disp, length; /* island::index, status, disp; history entries held */
  double at_time[PHN_TRACK_HISTORY], center[PHN_TRACK_HISTORY], volume[PHN_TRACK_HISTORY];
  double pot_en[PHN_TRACK_HISTORY], kin_en[PHN_TRACK_HISTORY], grad_en[PHN_TRACK_HISTORY];
  double av_phi[PHN_TRACK_HISTORY], peak_value[PHN_TRACK_HISTORY];
} phn_track_island;
enum {
  PHN_TRACK_ALIVE = 0,   /* found_islands after the last update, in its order */
  PHN_TRACK_RETIRED = 1, /* islands Old_islands removed in the last update (their history as written) */
  PHN_TRACK_BUBBLES = 2  /* islands print_bubble_history reported in the last update */
};
typedef struct phn_tracker phn_tracker;
int phn_tracker_create(int rank, phn_tracker **out);
int phn_tracker_destroy(phn_tracker *t);
int phn_tracker_reset(phn_tracker *t);
/* Full_Analysis on the handle's current state (Nc = 1): phn_islands with
 * (thres, mode, z_periodic), centre lookups, the bookkeeping below; labels
 * (optional, reference layout) receive island_analysis::b, the position of
 * each site's island in found_islands, -1 elsewhere. */
int phn_tracker_update(phn_tracker *t, phn_handle *h, double thres, int mode, int z_periodic, int *labels);
/* The bookkeeping alone, for callers that label islands themselves: comps[c]
 * are this update's islands in seed order, center_island[i] the island that
 * holds alive island i's centre (-1: outside the mask), in the current
 * found_islands order (phn_tracker_centers).  owner (optional, ncomp
 * entries) receives each island's position in found_islands afterwards. */
int phn_tracker_update_records(phn_tracker *t, double tau, const phn_island *comps, int ncomp,
                               const int *center_island, int *owner);
/* Centres (reference-layout index of the last entry) of the alive islands. */
int phn_tracker_centers(const phn_tracker *t, long long *pos, int max, int *n);
int phn_tracker_count(const phn_tracker *t, int set, int *n);
int phn_tracker_get(const phn_tracker *t, int set, int i, phn_track_island *out);
/* Oscillon_specific_observables (islands.cpp:745-775): over alive islands
 * with disp set and is_oscillon, out[0] = r_osc (their energy / (L^3
 * avg_energy), L = N a), out[1] = n_osc (count / L^3), out[2] = avgM_osc
 * (mean energy). */
int phn_tracker_oscillons(const phn_tracker *t, int N, double a, double avg_energy, double out[3]);
/* add_stat_new (statistics.cpp:43-67): adds the alive disp islands to the
 * 200 x 200 histograms of (|peak|, radius) and (|peak|, radius /
 * sqrt(log(peak^2 / thres^2))), row-major int counts. */
int phn_tracker_add_stat(const phn_tracker *t, double thres, double QS, int *hist_r, int *hist_r0);

/* Kernel path of the FP32 step (the others have one path each):
 * PHN_PATH_TMA, the TMA-pipelined persistent kernel (default where it
 * applies: Nc = 1, N in {128,256,384,512,768,1024}); PHN_PATH_X4, the
 * register kernel with four x-sites per thread (Nc = 1, N a multiple of 32);
 * or PHN_PATH_PLAIN, the register z-marching kernel (every size).  All compute
 * bit-identical fields.  PHN_PATH_AUTO restores the default. */
enum { PHN_PATH_AUTO = 0, PHN_PATH_PLAIN = 1, PHN_PATH_TMA = 2, PHN_PATH_X4 = 3 };
int phn_set_path(phn_handle *h, int path);
int phn_get_path(const phn_handle *h, int *path);

/* Autotuner of the FP32 and compensated FP32 steps: times the plain kernel
 * and every variant of the TMA kernel (FP32 only: tile height, stage count,
 * pi through shared memory or straight from HBM, grid policy) and of the x4
 * kernel (block shape, planes per item, grid policy) that applies to this
 * lattice, `steps` launches each on the live lattice, and keeps the fastest
 * for this handle.  *variant is its index (as phn_set_variant takes it) or -1
 * for the plain kernel.  The lattice state is unchanged; all kernels of a
 * precision compute bit-identical fields.  FP64 has one kernel: nothing to
 * tune (*variant = -1). */
int phn_autotune(phn_handle *h, int steps, int *variant, double *best_ms);
/* Number of variants on this handle -- the TMA kernel's first, then the x4
 * kernel's; 0 when neither applies -- and an explicit choice of one
 * (0 .. n-1, which also selects its path), e.g. to reproduce a tuned
 * configuration. */
int phn_num_variants(const phn_handle *h, int *n);
int phn_set_variant(phn_handle *h, int variant);

/* Self-test of the failure path: a kernel waits on a device barrier that
 * nothing completes, with a budget of `polls` polls (1 .. the step kernels'
 * budget), gives up, records the code in the handle's error word and returns.
 * Returns PHN_ERR_TIMEOUT, as a step whose pipeline stalled would; the handle
 * stays usable.  No copy is issued and nothing faults. */
int phn_wait_selftest(phn_handle *h, long long polls);

/* Self-test of the FP64 kernels' division by a constant (a multiply by a
 * one- or two-word reciprocal, then one residual correction): n operands a
 * drawn on the device
 * from `seed` -- half with random significands and exponents in
 * [2^-1000, 2^1000], half placed at ±1-2 ulps around b times a midpoint
 * between two doubles, plus zeros, subnormals, infinities and NaN -- each
 * divided by b both ways; *mismatches counts results whose bits differ from
 * IEEE a / b (NaN payloads aside).  n <= 2^34. */
int phn_divide_selftest(phn_handle *h, double b, long long n, unsigned long long seed, long long *mismatches);

/* Device pointers of the current fields (precision-typed: double* for
 * PHN_FP64, float* otherwise; SoA [a][z][y][x], no ghosts) and the stream the
 * handle launches on, for callers that keep data resident on the device. */
int phn_device_fields(phn_handle *h, void **phi, void **pi, void **stream);
int phn_synchronize(phn_handle *h);

/* Launch statistics: kernels launched by this handle since creation, and the
 * device time of the last phn_evolve / phn_run_loop step kernels (CUDA events
 * on the handle's stream), for roofline accounting. */
int phn_stats(const phn_handle *h, long long *kernel_launches, double *last_evolve_ms, int *last_evolve_steps);

/* ---- Batched ensemble ---------------------------------------------------
 * Many independent lattices (the reference run once per realization, one
 * `main` per seed) evolved together: one persistent kernel per step walks a
 * work list of (member, tile) items, and the step loop runs as a captured CUDA
 * graph.  Members: FP32, Nc = 1, N a multiple of 32, theory 0 or 1 with any
 * couplings; they share a, dt, T0 and the box (all static, or all expanding
 * with one H0): one clock, whose kick factor, drift factor and scale factor
 * per step the graph reads from a device table.  A member's fields are
 * bit-identical to those of a single-lattice handle with the same inputs. */
typedef struct phn_ensemble phn_ensemble;
int phn_ensemble_create(const phn_params *members, int n, phn_ensemble **out);
int phn_ensemble_destroy(phn_ensemble *e);
/* per member, reference layout as phn_upload / phn_download */
int phn_ensemble_upload(phn_ensemble *e, int member, const double *Phi, const double *Pi);
int phn_ensemble_download(phn_ensemble *e, int member, double *Phi, double *Pi);
/* reset() / n x evolve() for every member (dynamics.cpp:28-237) */
int phn_ensemble_reset(phn_ensemble *e);
int phn_ensemble_evolve(phn_ensemble *e, int nsteps);
int phn_ensemble_time(const phn_ensemble *e, double *tau, int *total_stepcount);
/* CalculateVolumeAverages + CalculateExtrema of every member: out[n] */
int phn_ensemble_averages(phn_ensemble *e, phn_averages *out);
/* phn_islands on one member */
int phn_ensemble_islands(phn_ensemble *e, int member, double thres, int mode, int z_periodic, int *labels,
                         phn_island *out, int max_out, int *n_islands);
/* Autotuner of the work-list tile (rows x planes per item): times every
 * candidate on the live ensemble (state unchanged) and keeps the fastest. */
int phn_ensemble_autotune(phn_ensemble *e, int steps, int *tile, double *best_ms);
int phn_ensemble_set_tile(phn_ensemble *e, int tile);
int phn_ensemble_stats(const phn_ensemble *e, long long *kernel_launches, double *last_evolve_ms,
                       int *last_evolve_steps);

/* ---- Adjoint ---------------------------------------------------------------
 * No counterpart in the reference (it has no derivatives).  Objective on the
 * final state: J = sum_x rho(x) sigmoid((rho(x) - 2 <rho>) / width), rho the
 * energy density (the summand of the reference's Energy), so width is in the
 * reference's energy units (Phi = sqrt(6) phi makes them 6x the units of the
 * phi^2/2 - phi^4/4 + g phi^6/6 form: its width 0.1 is 0.6 here).  Forward: the same
 * step kernels as phn_evolve, checkpoints every `every` steps.  Backward: the
 * discrete adjoint of the implemented leapfrog, reverse time stepping that
 * restarts from each checkpoint (finite-precision reversal drifts).
 * Theory 0 or 1, Nc = 1, static or expanding box, FP32 or FP64 (the FP64
 * run is the reference gradient).  In the expanding box rho carries the
 * kinetic terms of fieldanalysis.cpp:626-629 and the couplings at the final
 * scale factor, each reverse step the couplings of its kick; dJ/dc6 and dJ/dh
 * stay derivatives by the unscaled couplings. */
typedef struct phn_adjoint phn_adjoint;
int phn_adjoint_create(const phn_params *params, int nsteps, int every, double width, phn_adjoint **out);
int phn_adjoint_destroy(phn_adjoint *a);
/* reset() + nsteps x evolve() from (Phi0, Pi0) (reference layout); *J = J. */
int phn_adjoint_forward(phn_adjoint *a, const double *Phi0, const double *Pi0, double *J);
/* After a forward: dJ/dPhi0 and dJ/dPi0 in the reference layout (either may be
 * NULL; Pi0's ghost slabs untouched) and grads[3] = { dJ/d(homogeneous shift
 * of Phi0), dJ/dc6 with c6 = 1/(720 Kappa^2) the phi^6 coefficient of V
 * (theory 0), dJ/dh (theory 1) }. */
int phn_adjoint_backward(phn_adjoint *a, double *dPhi0, double *dPi0, double *grads);
/* Precision of the forward solve of an FP32 adjoint: PHN_FP64 runs the
 * forward with the FP64 step kernels (FP32 checkpoints, rounded; J and the
 * seed on the FP64 final state), the reverse sweep staying FP32; PHN_FP32_PAIR
 * runs it in FP32 pairs (double-float arithmetic for the force, the
 * increments and the updates; FP32 checkpoints; J and the seed on the pair
 * state widened to FP64) at FP32-pipe speed; PHN_FP32 (the default) runs
 * both in FP32.  The gradient's sensitivity to the final state through the
 * sigmoid makes the forward's precision the one that matters.
 * PHN_ERR_UNSUPPORTED for an FP64 adjoint or other precisions. */
int phn_adjoint_set_forward_precision(phn_adjoint *a, int precision);
/* J of the last forward and device times (ms) of the last forward and backward. */
int phn_adjoint_info(const phn_adjoint *a, double *J, double *forward_ms, double *backward_ms);

/* Volume averages of caller-owned device fields, allocating nothing.
 * No counterpart in the reference: it exists for hosts that cannot allocate
 * device memory where they need the averages -- a framework that owns all
 * device memory through its own pool, or a stream-ordered loop in which a
 * cudaMalloc (which may synchronise the device) is not allowed.
 * d_phi, d_pi: device fields in the layout phn_device_fields describes
 * (PHN_FP64: double, PHN_FP32: float; PHN_FP32_KAHAN is rejected); stream:
 * the cudaStream_t to run on (NULL: the legacy default stream); out: host.
 * The reduction's scratch is one fixed __device__ array of 768 KiB per GPU
 * (kept until the process exits), which limits N to 1024; larger lattices
 * get PHN_ERR_INVALID.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress); make that first call before any
 * stream capture.  The address is kept with the ID of the CUDA context it
 * belongs to and looked up again when the calling thread's current context
 * is another one (after the device was reset, or under a context the host
 * created with the driver API), so such a call is a set-up call too.  All
 * calls share the array: calls that overlap on the GPU race, so serialise
 * them.  The call synchronises `stream` and returns after the result is on
 * the host.  out->t is T0: the fields are taken as the state at tau = T0, and
 * the expanding box's averages use that time's scale factor
 * sqrt(1 + 2 H_0 T0). */
int phn_volume_averages_noalloc(const phn_params *params, const void *d_phi, const void *d_pi, void *stream,
                                phn_averages *out);

/* Page-locks (unlocks) a caller-owned host buffer so that phn_upload /
 * phn_download move it by DMA at full link bandwidth (cudaHostRegister). */
int phn_pin_host(void *ptr, size_t bytes);
int phn_unpin_host(void *ptr);

#ifdef __cplusplus
}
#endif
#endif

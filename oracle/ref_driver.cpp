/*
 * Oracle pin: PhiNum's own hot-path sources, compiled UNCHANGED from the
 * reference tree against the single-rank shims in oracle/ref_shim/, behind a
 * small extern "C" surface that the golden-vector generator
 * (tests/golden/make_golden.py) drives through ctypes.
 *
 * TEST INFRASTRUCTURE ONLY.  The result (oracle/_ref/libphinum_ref_*.so) is
 * built by oracle/build_ref.sh in a container that holds the reference tree;
 * it is never shipped, never linked into the product and never timed.
 *
 * What this file supplies in place of the reference's main.cpp and
 * parameters.cpp:
 *   - the parameter block (parameters.cpp:7-303 declares these names as
 *     compile-time switches plus globals; the names must match because the
 *     reference functions use them directly).  `theory` and `doubleprecision`
 *     come from -DPHN_REF_THEORY / -DPHN_REF_PRECISION so that one recipe
 *     builds every variant without editing a reference file;
 *   - the run loop of main.cpp:685-699 with an explicit step count in place
 *     of `tau < TMax` (an accumulated FP sum), and without the island,
 *     false-vacuum and spectrum calls, which are exposed separately.
 */
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <queue>
#include <vector>
#include <algorithm>
#include <sys/stat.h>

#include "mpi.h"
#include "fftw3-mpi.h"

using namespace std;

#include "ref_params.h"

/* ---- the reference's own hot-path sources, unchanged ----------------------- */
#include "lattice.cpp"
#include "util.cpp"
#include "comm.cpp"
#include "dynamics.cpp"
#include "fieldanalysis.cpp"
#include "clusterfft.cpp"
#include "momentumspace.cpp"
#include "islands.cpp"
#include "renormalization.cpp"

/* SetInitialConditions seeds with srand48(time(NULL)*(ID+1))
 * (initialconditions.cpp:16).  While its source is included, `time` names a
 * function returning a seed the harness chooses, so the stream is
 * reproducible; the file itself is compiled unchanged. */
static long g_ref_seed = 0;
static time_t phn_ref_seed_clock(time_t *) { return (time_t)g_ref_seed; }
#define time(x) phn_ref_seed_clock(x)
#include "initialconditions.cpp"
#undef time
#include "filter.cpp"

/* ---- extern "C" surface for the golden-vector generator -------------------- */
namespace {
bool g_ready = false;
size_t field_len() { return (size_t)Nc * N_t * N_t * (LocalLattice::N_eta_loc + 2); }
}

extern "C" {

/* Layout of the averages record written by ref_averages / ref_run_loop. */
enum { REF_MAX_NC = 4, REF_AVG_LEN = 1 + 2 * REF_MAX_NC + 14 + 3 };

int ref_precision() { return doubleprecision; }
int ref_theory() { return theory; }

/* H_0 of the expanding box (parameters.cpp:177); call before ref_init. */
void ref_set_h0(double h0) { H_0 = (pseudo_double)h0; }

/* Conformal time and scale factor (lattice.cpp:14-17); the static box gives
 * tau and 1. */
void ref_expansion_state(double *tau_c, double *a) {
#if (expansion == 1)
  *tau_c = (double)LocalLattice::tau_conformal;
  *a = (double)LocalLattice::scale_factor;
#else
  *tau_c = (double)LocalLattice::tau;
  *a = 1.0;
#endif
}

/* Couplings of theories 3-5 (M_mono_sqr, g, p_mono); call before ref_init. */
void ref_set_extra(double gcub, double pmono, double mmono) {
  g = (pseudo_double)gcub;
  p_mono = (pseudo_double)pmono;
  M_mono_sqr = (pseudo_double)mmono;
}

int ref_init(int N, int nc, double a, double dt, double t0, int mass_mode, double m_sqr,
             int lambda_mode, double lambda, double kappa, double hlin) {
  if (g_ready) return -1;
  if (nc < 1 || nc > REF_MAX_NC) return -2;
  N_t = N;
  Nc = nc;
  a_t = (pseudo_double)a;
  dtBaseLong = (pseudo_double)dt;
  T0 = (pseudo_double)t0;
  Mass_Mode = mass_mode;
  M_sqr = (pseudo_double)m_sqr;
  Lambda_Mode = lambda_mode;
  Lambda = (pseudo_double)lambda;
  Kappa = (pseudo_double)kappa;
  h = (pseudo_double)hlin;
  /* CompleteParameters (parameters.cpp:398-411): cubic box, dt base */
  a_eta = a_t;
  N_eta = N_t;
  dtBaseTrans = dtBaseLong;
  LocalLattice::init();
  FFT::init();
  MomentumSpace::init();
  island_analysis::init();
  fix_tadpole();
  reset();
  g_ready = true;
  return 0;
}

void ref_fin() {
  if (!g_ready) return;
  island_analysis::fin();
  MomentumSpace::fin();
  FFT::fin();
  LocalLattice::fin();
  g_ready = false;
}

/* Fields in the reference layout Nc*N*N*(N+2) (ghost z-slabs 0 and N+1);
 * only the interior is read, then the ghosts are filled by exchange(). */
void ref_set_fields(const double *phi, const double *pi) {
  const size_t n = field_len();
  for (size_t k = 0; k < n; ++k) {
    LocalLattice::Phi[k] = (pseudo_double)phi[k];
    LocalLattice::Pi[k] = (pseudo_double)pi[k];
  }
  Communication::exchange();
}

void ref_get_fields(double *phi, double *pi) {
  const size_t n = field_len();
  for (size_t k = 0; k < n; ++k) {
    phi[k] = (double)LocalLattice::Phi[k];
    pi[k] = (double)LocalLattice::Pi[k];
  }
}

void ref_reset() { reset(); }

void ref_evolve(int nsteps) {
  for (int s = 0; s < nsteps; ++s) evolve();
}

void ref_time(double *tau, int *stepcount) {
  *tau = (double)LocalLattice::tau;
  *stepcount = numeric::total_stepcount;
}

static void record(double t, double *out) {
  using namespace LocalLattice;
  int i = 0;
  out[i++] = t;
  for (int a = 0; a < REF_MAX_NC; ++a) out[i++] = a < Nc ? (double)avgphi[a] : 0.0;
  for (int a = 0; a < REF_MAX_NC; ++a) out[i++] = a < Nc ? (double)avgpi[a] : 0.0;
  out[i++] = avgphi2;
  out[i++] = avgpi2;
  out[i++] = avgphipi;
  out[i++] = avgphi4;
  out[i++] = avgphi6;
  out[i++] = avgEnergy;
  out[i++] = avgInteraction;
  out[i++] = avgCharge;
  out[i++] = GlminPhi;
  out[i++] = GlmaxPhi;
  out[i++] = GlmaxAbsPhi;
  out[i++] = (double)minpos;
  out[i++] = (double)maxpos;
  out[i++] = (double)maxAbspos;
  out[i++] = 0.0;
  out[i++] = 0.0;
#if (expansion == 1)
  out[i++] = (double)scale_factor;  /* the SO row's scale-factor column (fieldanalysis.cpp:789-791) */
#else
  out[i++] = 1.0;
#endif
}

int ref_avg_len() { return REF_AVG_LEN; }

/* One CalculateExtrema + CalculateVolumeAverages pass on the current state. */
void ref_averages(double *out) {
  CalculateExtrema();
  CalculateVolumeAverages();
  record((double)LocalLattice::tau, out);
}

/* main.cpp:685-699 with an explicit step count: before every evolve() the
 * reference's own Print_AveragesExtrema() decides (TSO cadence on the
 * accumulated tau) whether to compute a row; each row computed is recorded.
 * Returns the number of rows written (at most max_rows). */
int ref_run_loop(int nsteps, double tso, double *rows, int max_rows) {
  TSO = (pseudo_double)tso;
  int nrows = 0;
  int count = 0;
  for (reset(); count < nsteps; evolve(), ++count) {
    const bool due = !(numeric::total_stepcount > 0 &&
                       LocalLattice::tau < numeric::LastSOoutput + TSO);
    Print_AveragesExtrema();
    if (due && nrows < max_rows) {
      record((double)numeric::LastSOoutput, rows + (size_t)nrows * REF_AVG_LEN);
      ++nrows;
    }
  }
  return nrows;
}

/* The reference's false_vacuum_decayed() (fieldanalysis.cpp:887-893) on an
 * avgInteraction of v. */
int ref_false_vacuum_decayed(double v) {
  LocalLattice::avgInteraction = (pseudo_double)v;
  return false_vacuum_decayed() ? 1 : 0;
}

/* main.cpp:77-90 without islands and spectra, with an explicit step cap:
 * Print_AveragesExtrema(), then the false_vacuum_decayed() break, then
 * evolve().  Rows as ref_run_loop; *stop receives total_stepcount when the
 * loop broke, -1 when it ran all nsteps. */
int ref_run_until_decayed(int nsteps, double tso, double *rows, int max_rows, int *stop) {
  TSO = (pseudo_double)tso;
  int nrows = 0;
  int count = 0;
  *stop = -1;
  for (reset(); count < nsteps; evolve(), ++count) {
    const bool due = !(numeric::total_stepcount > 0 &&
                       LocalLattice::tau < numeric::LastSOoutput + TSO);
    Print_AveragesExtrema();
    if (due && nrows < max_rows) {
      record((double)numeric::LastSOoutput, rows + (size_t)nrows * REF_AVG_LEN);
      ++nrows;
    }
    if (false_vacuum_decayed()) {
      *stop = numeric::total_stepcount;
      break;
    }
  }
  return nrows;
}

int ref_nbins() { return MomentumSpace::nTBins; }
double ref_binsize() { return (double)MomentumSpace::binsizeT; }

/* Calculate_CorrelationFunctions (momentumspace.cpp:140-278) on the current
 * fields; outputs TotalCorrF/K/Q[bin*Nc + a] and TotalBCounts[bin]. */
void ref_spectrum(double *F, double *K, double *Q, int *counts) {
  Calculate_CorrelationFunctions();
  for (int k = 0; k < MomentumSpace::nTBins * Nc; ++k) {
    F[k] = (double)MomentumSpace::TotalCorrF[k];
    K[k] = (double)MomentumSpace::TotalCorrK[k];
    Q[k] = (double)MomentumSpace::TotalCorrQ[k];
  }
  for (int k = 0; k < MomentumSpace::nTBins; ++k) counts[k] = MomentumSpace::TotalBCounts[k];
}

/* The threshold the last Full_Analysis used: the caller's, or with
 * EnergybasedID 4 <rho> (islands.cpp:783-786). */
double ref_island_thres() { return (double)island_analysis::thres; }

#if (withEnergyPS == 1)
/* CalculateVolumeAverages (fieldanalysis.cpp:399-699) on the current fields
 * and its per-site energy density Delta (fieldanalysis.cpp:446-560), the
 * reference layout's interior. */
void ref_delta(double *out) {
  CalculateVolumeAverages();
  const size_t slab = (size_t)Nc * N_t * N_t;
  for (size_t k = 0; k < slab * (size_t)LocalLattice::N_eta_loc; ++k) out[k] = (double)LocalLattice::Delta[slab + k];
}

/* After ref_spectrum: TotalCorrD[bin*Nc + a], the binned power of the
 * density contrast (momentumspace.cpp:165-183, 233-270). */
void ref_spectrum_d(double *D) {
  for (int k = 0; k < MomentumSpace::nTBins * Nc; ++k) D[k] = (double)MomentumSpace::TotalCorrD[k];
}
#endif

/* One Full_Analysis (islands.cpp:778-840) from an empty island history with
 * the given threshold.  labels[] receives the reference's b[] array (the
 * reference layout, -1 outside islands); stats[i*8 + ...] = index, V, PotEn,
 * KinEn, GradEn, avPhi, peak position, Peak_value for each island found, in
 * the reference's found_islands order.  Returns the island count. */
int ref_islands(double thres, int *labels, double *stats, int max_islands) {
  using namespace island_analysis;
  island_analysis::fin();
  island_analysis::init();
  island_analysis::thres = (pseudo_double)thres;
  Full_Analysis();
  const size_t n = field_len();
  for (size_t k = 0; k < n; ++k) labels[k] = b[k];
  const int count = (int)found_islands.size();
  for (int i = 0; i < count && i < max_islands; ++i) {
    island &B = found_islands[(size_t)i];
    double *s = stats + (size_t)i * 8;
    s[0] = (double)B.index;
    s[1] = (double)B.V.back();
    s[2] = (double)B.PotEn.back();
    s[3] = (double)B.KinEn.back();
    s[4] = (double)B.GradEn.back();
    s[5] = (double)B.avPhi.back();
    s[6] = (double)B.center.back().pos;
    s[7] = (double)B.Peak_value.back();
  }
  return count;
}

/* Island tracking over a run: ref_track_reset() empties the history, then
 * each ref_track_step(thres) runs the reference's Full_Analysis() on the
 * current fields (islands.cpp:778-840: sort, Old_islands, re-seeding from
 * the old centres, new islands) and returns the number of tracked islands;
 * ref_track_island(i, out) reports island i as
 *   out[0..3]   index, status, disp, history length L (<= 5)
 *   out[4 + 8 j .. 11 + 8 j], j < L: at_time, centre pos, V, PotEn, KinEn,
 *               GradEn, avPhi, Peak_value of history entry j. */
void ref_track_reset() {
  island_analysis::fin();
  island_analysis::init();
}

int ref_track_step(double thres, int *labels) {
  using namespace island_analysis;
  island_analysis::thres = (pseudo_double)thres;
  Full_Analysis();
  if (labels) {
    const size_t n = field_len();
    for (size_t k = 0; k < n; ++k) labels[k] = b[k];
  }
  return (int)found_islands.size();
}

int ref_track_island(int i, double *out) {
  using namespace island_analysis;
  if (i < 0 || i >= (int)found_islands.size()) return -1;
  island &B = found_islands[(size_t)i];
  const int L = (int)B.V.size();
  out[0] = B.index;
  out[1] = B.status;
  out[2] = B.disp ? 1.0 : 0.0;
  out[3] = L;
  for (int j = 0; j < L && j < 5; ++j) {
    double *e = out + 4 + 8 * j;
    e[0] = B.at_time[(size_t)j];
    e[1] = B.center[(size_t)j].pos;
    e[2] = B.V[(size_t)j];
    e[3] = B.PotEn[(size_t)j];
    e[4] = B.KinEn[(size_t)j];
    e[5] = B.GradEn[(size_t)j];
    e[6] = B.avPhi[(size_t)j];
    e[7] = B.Peak_value[(size_t)j];
  }
  return L;
}

/* apply_filter(r, which) (filter.cpp:53-133) on the current fields; for
 * which = 2 the table W_import[0..n) and dp_import are set first (the
 * reference reads them from bounce.txt, filter.cpp:32-44). */
int ref_apply_filter(double r, int which, const double *table, int n, double dp) {
  if (which == 2) {
    if (!table || n < 1 || n > 25000) return -1;
    for (int i = 0; i < 25000; ++i) ImportFilter::W_import[i] = (pseudo_double)table[i < n ? i : n - 1];
    ImportFilter::dp_import = (pseudo_double)dp;
  }
  apply_filter((pseudo_double)r, which);
  return 0;
}

/* SaveConfig(Name) (fieldanalysis.cpp:252-283): writes ./field-<name>-0.out
 * and ./moment-<name>.out in the working directory. */
void ref_save_config(int name) { SaveConfig(name); }

/* The globals of initialize 0-2 and 4 (parameters.cpp:207-272): chi,
 * FAmp, Lambda, Temperature and the homogeneous phi0, pi0 of component 0. */
void ref_set_ic_extra(double chi_, double famp, double lambda, double temperature, double phi0_, double pi0_) {
  chi = (pseudo_double)chi_;
  FAmp = (pseudo_double)famp;
  Lambda = (pseudo_double)lambda;
  Temperature = (pseudo_double)temperature;
  phi0 = (pseudo_double)phi0_;
  pi0 = (pseudo_double)pi0_;
}

/* SetInitialConditions() (the build's `initialize` and `withcharge`) with
 * srand48(seed); the fields land in LocalLattice::Phi/Pi (read them with
 * ref_get_fields). */
int ref_initial_conditions(long seed, int justnoise_, double qs, double scale2_, double amplitude, double noise,
                           double phi00, double phi01, double pi00, double pi01) {
  if (!g_ready) return -1;
  g_ref_seed = seed;
  justnoise = justnoise_;
  QS = (pseudo_double)qs;
  scale2 = (pseudo_double)scale2_;
  Amplitude = (pseudo_double)amplitude;
  Noise = (pseudo_double)noise;
  phi0_0 = (pseudo_double)phi00;
  phi0_1 = (pseudo_double)phi01;
  pi0_0 = (pseudo_double)pi00;
  pi0_1 = (pseudo_double)pi01;
  randGen::on = 0;
  SetInitialConditions();
  return 0;
}

} /* extern "C" */

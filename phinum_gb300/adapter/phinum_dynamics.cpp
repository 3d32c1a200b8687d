// phinum_dynamics.cpp -- the reference host's side of the GPU drop-in.
//
// Included by PhiNum's main.cpp after its own sources (the reference builds as
// one translation unit, main.cpp:8-20).  It replaces, for the run loop of
// main.cpp:685-699, the hot-path entry points with versions backed by
// libphinum_gpu (include/phinum_gpu.h), writing their results into the
// reference's own globals so that every printer and check downstream is
// unchanged:
//
//   reference (file:line)                          here
//   reset()            dynamics.cpp:28-50          phn_gpu::reset()
//   evolve()           dynamics.cpp:196-237        phn_gpu::evolve()
//   Print_AveragesExtrema  fieldanalysis.cpp:748-799  phn_gpu::Print_AveragesExtrema()
//     (CalculateExtrema :319, CalculateVolumeAverages :399)
//   Print_fp           momentumspace.cpp:280-384   phn_gpu::Print_fp()
//     (Calculate_CorrelationFunctions :140)
//   Full_Analysis      islands.cpp:778-840         phn_gpu::Full_Analysis_first()
//     (first call of a run: empty island history), or phn_gpu::Full_Analysis()
//     for every call with the history (islands.cpp:651-840)
//
// The device holds the authoritative fields between calls; phn_gpu::to_host()
// brings them back into LocalLattice::Phi/Pi for any host code that reads
// them directly (SaveConfig, visualisation).  Theories 0-5, static or
// expanding box (expansion 0 or 1), FP64 by default (bit-identical to the CPU
// build for theories 0, 1 and 4) or FP32 with PHN_PRECISION=1 in the
// environment.
#ifndef PHINUM_DYNAMICS_ADAPTER_CPP
#define PHINUM_DYNAMICS_ADAPTER_CPP

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "phinum_gpu.h"

#if (withEnergyPS == 1)
#error "phinum_gpu adapter: withEnergyPS 1 (the energy spectrum and EnergybasedID) has no GPU drop-in"
#endif

namespace phn_gpu {

static phn_handle *handle = nullptr;

static void check(int status, const char *what) {
  if (status != PHN_OK) {
    std::fprintf(stderr, "phinum_gpu: %s failed (%d): %s\n", what, status, phn_last_error());
    std::exit(1);
  }
}

// LocalLattice::Phi/Pi transfers in the build's pseudo_double: double
// (doubleprecision 0) or float (doubleprecision -1).
static void upload(const double *Phi, const double *Pi) { check(phn_upload(handle, Phi, Pi), "phn_upload"); }
static void upload(const float *Phi, const float *Pi) { check(phn_upload_f32(handle, Phi, Pi), "phn_upload_f32"); }
static void download(double *Phi, double *Pi) { check(phn_download(handle, Phi, Pi), "phn_download"); }
static void download(float *Phi, float *Pi) { check(phn_download_f32(handle, Phi, Pi), "phn_download_f32"); }

// Mirrors the reference clock (LocalLattice::tau, numeric::Last_*_update,
// numeric::total_stepcount) from the handle after every call that moves it.
static void mirror_clock() {
  double tau = 0.0;
  int steps = 0;
  check(phn_time(handle, &tau, &steps), "phn_time");
  LocalLattice::tau = tau;
  LocalLattice::dtau = dtBaseTrans * a_t;
  numeric::Last_Field_update = tau;
  numeric::Last_Momenta_update = tau;
  numeric::total_stepcount = steps;
  numeric::normal_stepcount = steps;
#if (expansion == 1)
  double tau_c = 0.0, sf = 1.0;
  check(phn_conformal_time(handle, &tau_c, &sf), "phn_conformal_time");
  LocalLattice::tau_conformal = tau_c;
  LocalLattice::scale_factor = sf;
  numeric::Last_Field_update_conformal = tau_c;
  numeric::Last_Momenta_update_conformal = tau_c;
#endif
}

// After LocalLattice::init, fix_tadpole and SetInitialConditions: creates the
// device lattice from the reference's parameters and uploads Phi/Pi.  The
// device holds the whole lattice, so the run must be a single rank: with
// mpirun -np K > 1 each rank's Phi/Pi hold only its z-slab
// (Nc*N*N*(N_eta_loc+2) values, lattice.cpp:72-78) and are refused here
// rather than read past their end.
inline void init() {
  if (nodes != 1 || LocalLattice::N_eta_loc != N_eta || N_eta != N_t) {
    std::fprintf(stderr,
                 "phinum_gpu: the GPU drop-in evolves the whole %d^3 lattice on one rank; this run has %d "
                 "rank(s) holding %d of %d z-slabs each (run with one MPI rank)\n",
                 N_t, nodes, LocalLattice::N_eta_loc, N_eta);
    std::exit(1);
  }
  phn_params p;
  std::memset(&p, 0, sizeof(p));
  p.N = N_t;
  p.Nc = Nc;
  // the couplings each theory defines (parameters.cpp:86-170)
#if (theory == 0)
  p.potential = 0;
  p.kappa = Kappa;
  p.mass_mode = Mass_Mode;
  p.lambda_mode = Lambda_Mode;
#elif (theory == 1)
  p.potential = 1;
  p.h = ::h;  // the reference's linear coupling (parameters.cpp:117)
  p.mass_mode = Mass_Mode;
  p.lambda_mode = Lambda_Mode;
#elif (theory == 2)
  p.potential = 2;
#elif (theory == 3)
  p.potential = 3;
  p.m_mono_sqr = LocalLattice::BareM_mono_sqr_long;
#elif (theory == 4)
  p.potential = 4;
  p.g = ::g;
  p.mass_mode = Mass_Mode;
  p.lambda_mode = Lambda_Mode;
#elif (theory == 5)
  p.potential = 5;
  p.p_mono = ::p_mono;
#endif
  p.m_sqr = LocalLattice::BareM_sqr_long;
  p.a = a_t;
  p.dt = dtBaseTrans;
  p.T0 = T0;
#if (expansion == 1)
  p.expanding = 1;  // radiation-era box (dynamics.cpp:36-50)
  p.H0 = H_0;
#endif
  const char *prec = std::getenv("PHN_PRECISION");
  p.precision = prec ? std::atoi(prec) : PHN_FP64;
  if (handle) phn_destroy(handle);
  check(phn_create(&p, &handle), "phn_create");
  upload(LocalLattice::Phi, LocalLattice::Pi);
}

inline void fin() {
  if (handle) phn_destroy(handle);
  handle = nullptr;
}

// Brings the device fields back into LocalLattice::Phi/Pi.
inline void to_host() { download(LocalLattice::Phi, LocalLattice::Pi); }

// reset() (dynamics.cpp:28-50).
inline void reset() {
  numeric::regime = 0;
  numeric::adaptive_stepcount = 0;
  check(phn_reset(handle), "phn_reset");
  mirror_clock();
}

// evolve() (dynamics.cpp:196-237): kick, drift and halo in one kernel.
inline void evolve() {
  check(phn_evolve(handle, 1), "phn_evolve");
  mirror_clock();
}

// Copies one averages record into the reference's globals (lattice.cpp:44-58).
static void store_averages(const phn_averages &a) {
  using namespace LocalLattice;
  for (int c = 0; c < Nc && c < PHN_MAX_NC; ++c) {
    avgphi[c] = a.phi[c];
    avgpi[c] = a.pi[c];
  }
  avgphi2 = a.phi2;
  avgpi2 = a.pi2;
  avgphipi = a.phipi;
  avgphi4 = a.phi4;
  avgphi6 = a.phi6;
  avgEnergy = a.energy;
  avgInteraction = a.interaction;
  avgCharge = a.charge;
  GlminPhi = a.min_phi;
  GlmaxPhi = a.max_phi;
  GlmaxAbsPhi = a.max_abs_phi;
  minpos = (int)a.min_pos;
  maxpos = (int)a.max_pos;
  maxAbspos = (int)a.max_abs_pos;
  GlminID = GlmaxID = GlmaxAbsID = 0;
}

// CalculateExtrema() + CalculateVolumeAverages() on the device state.
inline void CalculateVolumeAverages() {
  phn_averages a;
  const int r = phn_volume_averages(handle, &a);
  if (r != PHN_OK && r != PHN_ERR_NONFINITE) check(r, "phn_volume_averages");
  store_averages(a);  // NaN reaches false_vacuum_decayed() as in the reference
}

// Print_AveragesExtrema() (fieldanalysis.cpp:748-799): same cadence, same row.
inline void Print_AveragesExtrema() {
  using namespace std;
  using namespace LocalLattice;
  if (numeric::total_stepcount > 0 && tau < numeric::LastSOoutput + TSO) return;
  if (numeric::total_stepcount == 0) {
    if (ID == 0) {
      if (runID > 1) SpatialObs.close();
      char fname[256];
      snprintf(fname, 256, "./output/%i/SO-%i.txt", LASTRUN, runID);
      SpatialObs.open(fname, fstream::app);
    }
    numeric::LastSOoutput = tau;
#if (expansion == 1)
    numeric::LastSOoutput_conformal = (sqrt(1. + 2. * H_0 * tau) - 1.) / H_0;
#endif
  } else if (tau >= numeric::LastSOoutput + TSO) {
    numeric::LastSOoutput += TSO;
#if (expansion == 1)
    numeric::LastSOoutput_conformal = (sqrt(1. + 2. * H_0 * numeric::LastSOoutput) - 1.) / H_0;
#endif
  }
  CalculateVolumeAverages();
  if (ID == 0) {
#if (expansion == 1)
    SpatialObs << scale_factor << ' ';  // the expanding box's time column (fieldanalysis.cpp:789-791)
#else
    SpatialObs << numeric::LastSOoutput << ' ';
#endif
    for (int i = 0; i < Nc; i++) SpatialObs << avgphi[i] << ' ' << avgpi[i] << ' ';
    SpatialObs << avgphi2 << ' ' << avgpi2 << ' ' << avgphipi << ' ' << avgphi4 << ' ' << avgphi6 << ' ';
    SpatialObs << avgEnergy << ' ' << avgInteraction << ' ' << avgCharge << ' ';
    SpatialObs << GlminPhi << ' ' << GlmaxPhi << ' ' << GlmaxAbsPhi << endl;
  }
}

// Calculate_CorrelationFunctions() into MomentumSpace::TotalCorrF/K/Q and
// TotalBCounts (momentumspace.cpp:140-278).
inline void Calculate_CorrelationFunctions() {
  using namespace MomentumSpace;
  int nb = 0;
  double bs = 0.0;
  check(phn_spectrum_bins(handle, &nb, &bs), "phn_spectrum_bins");
  std::vector<double> F((size_t)nb * Nc), K((size_t)nb * Nc), Q((size_t)nb * Nc);
  std::vector<int> C((size_t)nb);
  check(phn_spectrum(handle, F.data(), K.data(), Q.data(), C.data(), nb), "phn_spectrum");
  for (int k = 0; k < nTBins && k < nb; ++k) {
    TotalBCounts[k] = C[(size_t)k];
    for (int a = 0; a < Nc; ++a) {
      TotalCorrF[k * Nc + a] = F[(size_t)k * Nc + a];
      TotalCorrK[k * Nc + a] = K[(size_t)k * Nc + a];
      TotalCorrQ[k * Nc + a] = Q[(size_t)k * Nc + a];
    }
  }
}

// Print_fp() (momentumspace.cpp:280-384): same cadence; the spectrum comes
// from the device and the Distrib-<run>-<t>.txt file gets the same columns as
// the reference's printer (momentumspace.cpp:307-381), the expanding box's
// scale factor included (:363-365).  The energy spectrum columns of
// withEnergyPS 1 (:366-371) have no device counterpart: that switch is
// refused at compile time below.
inline void Print_fp() {
  using namespace LocalLattice;
  if (numeric::total_stepcount > 0 && tau < numeric::LastMOoutput + TMO) return;
  if (numeric::total_stepcount == 0) {
    numeric::LastMOoutput = tau;
#if (expansion == 1)
    numeric::LastMOoutput_conformal = (sqrt(1. + 2. * H_0 * tau) - 1.) / H_0;
#endif
  } else if (tau >= numeric::LastMOoutput + TMO) {
    numeric::LastMOoutput += TMO;
#if (expansion == 1)
    numeric::LastMOoutput_conformal = (sqrt(1. + 2. * H_0 * numeric::LastMOoutput) - 1.) / H_0;
#endif
  }
  Calculate_CorrelationFunctions();
  if (ID == 0) {
    using namespace MomentumSpace;
    std::ofstream specOut;
    char fname[256];
    snprintf(fname, 256, "./output/%i/Distrib-%i-%g.txt", LASTRUN, runID, really_double(numeric::LastMOoutput));
    specOut.open(fname);
    // the printer's locals are pseudo_double, as the reference declares them,
    // so the single-precision build rounds and prints as it does
    const pseudo_double NormCorr = 1. / (sqr(N_t * a_t) * N_eta * a_eta);
    for (int k = 0; k < nTBins; k++) {
      const pseudo_double norm2 = (TotalBCounts[k] == 0 ? 0 : 1 / (pseudo_double)(TotalBCounts[k]));
      const pseudo_double pabs = binsizeT * k;
      if (norm2 != 0 && TotalCorrF[k * Nc] != 0) {
        if (k != 0) specOut << std::endl;
        specOut << pabs << " " << TotalBCounts[k] << " ";
        pseudo_double FF = 0, KK = 0, QQ = 0;
        for (int a = 0; a < Nc; a++) {
          FF += TotalCorrF[k * Nc + a];
          KK += TotalCorrK[k * Nc + a];
          QQ += TotalCorrQ[k * Nc + a];
        }
        FF /= Nc;
        KK /= Nc;
        QQ /= Nc;
        const pseudo_double omg = sqrt(KK / FF);
        specOut << omg << ' ' << FF * NormCorr * norm2 << ' ' << KK * NormCorr * norm2 << ' '
                << sqrt(FF * KK) * NormCorr * norm2 << " ";
#if (expansion == 1)
        specOut << scale_factor << " ";  // the expanding box's scale-factor column
#endif
        specOut << FF * NormCorr * norm2 * pabs * pabs * pabs / 2. / acos(-1.) / acos(-1.) << ' ';
        if (FF * KK - QQ * QQ < 0) std::cout << "negative at " << k << std::endl;
      }
    }
    specOut.close();
  }
}

// The labelling pass of a first Full_Analysis() (islands.cpp:778-840, empty
// history): island_analysis::b receives the labels, found_islands one entry
// per island in the reference's seed order with its statistics.
inline void Full_Analysis_first() {
  using namespace island_analysis;
  int n = 0;
  check(phn_islands(handle, thres, PHN_ISLAND_REFERENCE, 0, nullptr, nullptr, 0, &n), "phn_islands (count)");
  std::vector<phn_island> rec((size_t)(n > 0 ? n : 1));
  check(phn_islands(handle, thres, PHN_ISLAND_REFERENCE, 0, b, rec.data(), n, &n), "phn_islands");
  found_islands.clear();
  for (int i = 0; i < n; ++i) {
    island B;
    point P;
    P.pos = (int)rec[(size_t)i].peak_pos;
    P.id = ID;
    B.center.push_back(P);
    B.PotEn.push_back(rec[(size_t)i].pot_en);
    B.KinEn.push_back(rec[(size_t)i].kin_en);
    B.GradEn.push_back(rec[(size_t)i].grad_en);
    B.avPhi.push_back(rec[(size_t)i].av_phi);
    B.V.push_back(rec[(size_t)i].volume);
    B.Peak_value.push_back(rec[(size_t)i].peak_value);
    B.addr.push_back(-1);
    B.addl.push_back(-1);
    B.at_time.push_back(LocalLattice::tau);
    B.index = number_of_islands + ID * 1000000;
    B.status = 0;
    B.disp = 1;
    number_of_islands++;
    found_islands.push_back(B);
  }
}

// Full_Analysis() with its history (islands.cpp:651-840) on the device
// fields: the tracker does the labelling and the bookkeeping; its islands are
// then mirrored into island_analysis::found_islands, so the reference's own
// consumers (add_stat_new, Oscillon_specific_observables, is_bubble,
// is_oscillon) read them unchanged, and the reference's own writers record
// what this update retired (Old_islands: non_critical_islands.txt,
// islands.txt) and which expanding bubbles it saw (print_bubble_history).
static phn_tracker *tracker = nullptr;

static island to_island(const phn_track_island &r) {
  island B;
  const int L = (int)r.length;
  for (int j = 0; j < L; ++j) {
    point P;
    P.pos = (int)r.center[j];
    P.id = ID;
    B.center.push_back(P);
    B.at_time.push_back(r.at_time[j]);
    B.V.push_back(r.volume[j]);
    B.PotEn.push_back(r.pot_en[j]);
    B.KinEn.push_back(r.kin_en[j]);
    B.GradEn.push_back(r.grad_en[j]);
    B.avPhi.push_back(r.av_phi[j]);
    B.Peak_value.push_back(r.peak_value[j]);
    B.addr.push_back(-1);
    B.addl.push_back(-1);
  }
  B.index = (int)r.index;
  B.status = (int)r.status;
  B.disp = r.disp != 0.0;
  return B;
}

static void mirror_set(int set, std::vector<island> &dst) {
  int n = 0;
  check(phn_tracker_count(tracker, set, &n), "phn_tracker_count");
  dst.clear();
  phn_track_island r;
  for (int i = 0; i < n; ++i) {
    check(phn_tracker_get(tracker, set, i, &r), "phn_tracker_get");
    dst.push_back(to_island(r));
  }
}

inline void Full_Analysis() {
  using namespace island_analysis;
  if (!tracker) check(phn_tracker_create(ID, &tracker), "phn_tracker_create");
  check(phn_tracker_update(tracker, handle, thres, PHN_ISLAND_REFERENCE, 0, b), "phn_tracker_update");
  // retired islands through the reference's Old_islands: their centres are
  // outside the mask, so the host copy of the fields is set to 0 there first
  mirror_set(PHN_TRACK_RETIRED, found_islands);
  if (!found_islands.empty()) {
    for (island &B : found_islands)
      for (int a = 0; a < Nc; ++a) {
        LocalLattice::Phi[B.center.back().pos + a] = 0;
        LocalLattice::Pi[B.center.back().pos + a] = 0;
      }
    Old_islands();
  }
  // bubbles reported this update, printed from their own records
  std::vector<island> bubbles;
  mirror_set(PHN_TRACK_BUBBLES, bubbles);
  for (island &B : bubbles) {
    found_islands.assign(1, B);
    print_bubble_history(0);
  }
  mirror_set(PHN_TRACK_ALIVE, found_islands);
}

}  // namespace phn_gpu

#endif

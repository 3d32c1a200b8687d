// Drives the reference-side adapter (phinum_gb300/adapter/phinum_dynamics.cpp)
// through the real library on a GPU, without the reference tree.
//
// TEST INFRASTRUCTURE (tests/test_gpu_adapter.py).  The adapter is written
// against the reference's globals; this file declares the ones it uses, with
// the reference's names and types (parameters.cpp, lattice.cpp:8-64,
// dynamics.cpp:8-24, fieldanalysis.cpp:14, momentumspace.cpp:14-28,
// islands.cpp:13-59), so that the adapter compiles unchanged.  The run is the
// reference's sequence (main.cpp:64-90): averages and island threshold,
// Full_Analysis's first labelling, then the loop of reset / Print_AveragesExtrema
// / false_vacuum_decayed / Print_fp / Full_Analysis every 5 steps / evolve.
// Fields come from phi.bin and pi.bin (reference layout, doubles); the SO and
// Distrib files go to ./output/1/ as the reference writes them, and one line
// per island analysis ("step count islands") to islands.txt.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>
#include <sys/stat.h>

using namespace std;

// ---- the reference's compile-time switches (parameters.cpp:7-84) ----
#define theory 0
#define expansion 0
#define withEnergyPS 0
#define pseudo_double double
#define really_double double

// ---- parameter globals (parameters.cpp:86-201) ----
int N_t = 16, N_eta = 16, Nc = 1, nodes = 1, ID = 0, runID = 1, LASTRUN = 1;
int Mass_Mode = 1, Lambda_Mode = -1;
pseudo_double a_t = 0.25, a_eta = 0.25, dtBaseTrans = 0.08, T0 = 0.0, TMax = 1.0, TSO = 0.2, TMO = 0.5;
pseudo_double M_sqr = 1.0, Kappa = 1.7320508075688772, h = 0.0, g = 2.0, p_mono = -0.5, H_0 = 0.0171156;

pseudo_double sqr(pseudo_double x) { return x * x; }  // util.cpp:20-23

std::ofstream SpatialObs;  // fieldanalysis.cpp:14

namespace LocalLattice {  // lattice.cpp:8-64
pseudo_double *Phi, *Pi;
pseudo_double tau, dtau, tau_conformal, scale_factor = 1.0;
int N_eta_loc;
pseudo_double *avgphi, *avgpi;
pseudo_double avgpi2, avgphi2, avgphi4, avgphi6, avgphipi, avgEnergy, avgInteraction, avgCharge;
pseudo_double GlmaxPhi, GlminPhi, GlmaxAbsPhi;
int maxpos, minpos, maxAbspos, GlmaxID, GlminID, GlmaxAbsID;
pseudo_double BareM_sqr_long, BareM_sqr_trans, BareM_mono_sqr_long;
}  // namespace LocalLattice

namespace numeric {  // dynamics.cpp:8-24
int total_stepcount, normal_stepcount, adaptive_stepcount, regime;
pseudo_double Last_Field_update, Last_Momenta_update, LastMOoutput, LastSOoutput;
pseudo_double Last_Field_update_conformal, Last_Momenta_update_conformal;
pseudo_double LastMOoutput_conformal, LastSOoutput_conformal;
}  // namespace numeric

namespace MomentumSpace {  // momentumspace.cpp:14-28 (filled by the adapter)
pseudo_double *TotalCorrF, *TotalCorrK, *TotalCorrQ;
int *TotalBCounts;
pseudo_double binsizeT;
int nTBins;
}  // namespace MomentumSpace

struct point {  // islands.cpp
  int pos, id;
};
struct island {  // islands.cpp:13-28
  int index;
  bool disp;
  vector<point> center;
  vector<pseudo_double> V, at_time, PotEn, KinEn, GradEn, avPhi, Peak_value;
  vector<int> addr, addl;
  int status;
};
namespace island_analysis {  // islands.cpp:36-59
pseudo_double thres;
int number_of_islands;
vector<island> found_islands;
int *b;
}  // namespace island_analysis

// The reference's writers of retired islands and expanding bubbles
// (islands.cpp:651-744) are file output outside the path; here they count.
static int g_retired_calls = 0, g_bubble_calls = 0;
void Old_islands() { g_retired_calls++; }
void print_bubble_history(int) { g_bubble_calls++; }

bool false_vacuum_decayed() {  // fieldanalysis.cpp:887-893, theory 0
  const pseudo_double v = LocalLattice::avgInteraction;
  return v < 0 || v != v || v * 0. != 0.;
}

#include "phinum_dynamics.cpp"

static void read_field(const char *path, pseudo_double *dst, size_t n) {
  FILE *f = std::fopen(path, "rb");
  if (!f || std::fread(dst, sizeof(pseudo_double), n, f) != n) {
    std::fprintf(stderr, "cannot read %s\n", path);
    std::exit(2);
  }
  std::fclose(f);
}

int main(int argc, char **argv) {
  for (int i = 1; i < argc; ++i) {
    std::string s(argv[i]);
    const size_t eq = s.find('=');
    if (eq == std::string::npos) return 2;
    const std::string k = s.substr(0, eq);
    const double v = std::atof(s.c_str() + eq + 1);
    if (k == "N") N_t = N_eta = (int)v;
    else if (k == "TMax") TMax = v;
    else if (k == "TSO") TSO = v;
    else if (k == "TMO") TMO = v;
    else if (k == "Kappa") Kappa = v;
    else return 2;
  }
  using namespace LocalLattice;
  N_eta_loc = N_eta;
  BareM_sqr_long = BareM_sqr_trans = M_sqr;
  const size_t n = (size_t)Nc * N_t * N_t * (N_eta + 2);
  Phi = new pseudo_double[n];
  Pi = new pseudo_double[n];
  avgphi = new pseudo_double[Nc];
  avgpi = new pseudo_double[Nc];
  read_field("phi.bin", Phi, n);
  read_field("pi.bin", Pi, n);
  // MomentumSpace::init (momentumspace.cpp:32-65): the bin count and width
  // the library reports, with the reference's arrays
  MomentumSpace::binsizeT = 2. / a_t * std::sin(std::acos(-1.) / N_t);
  MomentumSpace::nTBins = int(std::sqrt(12.) / a_t / MomentumSpace::binsizeT + 0.5) + 2;
  const int nb = MomentumSpace::nTBins;
  MomentumSpace::TotalCorrF = new pseudo_double[(size_t)nb * Nc];
  MomentumSpace::TotalCorrK = new pseudo_double[(size_t)nb * Nc];
  MomentumSpace::TotalCorrQ = new pseudo_double[(size_t)nb * Nc];
  MomentumSpace::TotalBCounts = new int[nb];
  island_analysis::b = new int[n];
  mkdir("output", 0755);
  mkdir("output/1", 0755);

  std::ofstream isl("islands.txt");
  phn_gpu::init();
  phn_gpu::CalculateVolumeAverages();
  island_analysis::thres = 2.57583 * std::sqrt(avgphi2);  // main.cpp:70
  phn_gpu::Full_Analysis_first();
  isl << 0 << ' ' << island_analysis::found_islands.size() << '\n';
  for (phn_gpu::reset(); tau < TMax; phn_gpu::evolve()) {
    phn_gpu::Print_AveragesExtrema();
    if (numeric::total_stepcount % 5 == 0) {  // main.cpp:81-84
      phn_gpu::Full_Analysis();
      isl << numeric::total_stepcount << ' ' << island_analysis::found_islands.size() << '\n';
    }
    if (false_vacuum_decayed()) break;
    phn_gpu::Print_fp();
  }
  phn_gpu::to_host();
  phn_gpu::fin();
  SpatialObs.close();
  std::ofstream fout("fields_after.bin", std::ios::binary);
  fout.write((const char *)Phi, (std::streamsize)(n * sizeof(pseudo_double)));
  std::printf("done steps=%d thres=%.17g\n", numeric::total_stepcount, (double)island_analysis::thres);
  return 0;
}

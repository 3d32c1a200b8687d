// Compile check of phinum_gb300/adapter/phinum_dynamics.cpp inside the
// reference's single translation unit (the reference sources come from the
// reference tree, the MPI/FFTW stand-ins and the parameter block from
// oracle/).  TEST INFRASTRUCTURE: compiled with -fsyntax-only by
// tests/test_adapter.py; never run.
#include <algorithm>
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
#include <sys/stat.h>

#include "mpi.h"
#include "fftw3-mpi.h"

using namespace std;

#include "ref_params.h"

#include "lattice.cpp"
#include "util.cpp"
#include "comm.cpp"
#include "dynamics.cpp"
#include "fieldanalysis.cpp"
#include "clusterfft.cpp"
#include "momentumspace.cpp"
#include "islands.cpp"
#include "renormalization.cpp"
#include "initialconditions.cpp"

#include "phinum_dynamics.cpp"

// The reference's run loop (main.cpp:660-699) with the GPU calls in place.
int main(int argc, char **argv) {
  MPI_Init(&argc, &argv);
  MPI::init();
  LocalLattice::init();
  FFT::init();
  MomentumSpace::init();
  for (runID = 1; runID <= runs; runID++) {
    fix_tadpole();
    island_analysis::init();
    SetInitialConditions();
    phn_gpu::init();
    phn_gpu::CalculateVolumeAverages();
    island_analysis::thres = 2.57583 * sqrt(LocalLattice::avgphi2);
    phn_gpu::Full_Analysis_first();
    for (phn_gpu::reset(); LocalLattice::tau < TMax; phn_gpu::evolve()) {
      phn_gpu::Print_AveragesExtrema();
      if (false_vacuum_decayed()) break;
      phn_gpu::Print_fp();
      if (numeric::total_stepcount % 5 == 0) phn_gpu::Full_Analysis();  // main.cpp:81-84
    }
    phn_gpu::to_host();
    phn_gpu::fin();
    island_analysis::fin();
  }
  MomentumSpace::fin();
  FFT::fin();
  LocalLattice::fin();
  MPI_Finalize();
  return 0;
}

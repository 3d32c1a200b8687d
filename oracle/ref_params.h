/*
 * Parameter block standing in for PhiNum's parameters.cpp (which fixes the
 * theory and precision with #defines and parses the command line): the same
 * names, as compile-time switches plus globals, so that the reference's own
 * sources compile against it for any theory/precision chosen with
 * -DPHN_REF_THEORY / -DPHN_REF_PRECISION.  Defaults follow
 * parameters.cpp:84-303.  TEST INFRASTRUCTURE (oracle pin, adapter check).
 */
#ifndef PHN_REF_PARAMS_H
#define PHN_REF_PARAMS_H
#define _PARAMETERS_CPP_

#ifndef PHN_REF_THEORY
#define PHN_REF_THEORY 0
#endif
#ifndef PHN_REF_PRECISION
#define PHN_REF_PRECISION 0
#endif

#define doubleprecision PHN_REF_PRECISION
#if (doubleprecision == -1)
#define pseudo_double float
#define MPI_PSEUDO_DOUBLE MPI_FLOAT
#define really_double double
#define p_fftw_complex fftwf_complex
#define p_fftw_plan fftwf_plan
#define p_fftw_mpi_init fftwf_mpi_init
#define p_fftw_mpi_local_size_3d fftwf_mpi_local_size_3d
#define p_fftw_alloc_real fftwf_alloc_real
#define p_fftw_alloc_complex fftwf_alloc_complex
#define p_fftw_mpi_plan_dft_r2c_3d fftwf_mpi_plan_dft_r2c_3d
#define p_fftw_mpi_plan_dft_c2r_3d fftwf_mpi_plan_dft_c2r_3d
#define p_fftw_destroy_plan fftwf_destroy_plan
#define p_fftw_execute fftwf_execute
#else
#define pseudo_double double
#define MPI_PSEUDO_DOUBLE MPI_DOUBLE
#define really_double double
#define p_fftw_complex fftw_complex
#define p_fftw_plan fftw_plan
#define p_fftw_mpi_init fftw_mpi_init
#define p_fftw_mpi_local_size_3d fftw_mpi_local_size_3d
#define p_fftw_alloc_real fftw_alloc_real
#define p_fftw_alloc_complex fftw_alloc_complex
#define p_fftw_mpi_plan_dft_r2c_3d fftw_mpi_plan_dft_r2c_3d
#define p_fftw_mpi_plan_dft_c2r_3d fftw_mpi_plan_dft_c2r_3d
#define p_fftw_destroy_plan fftw_destroy_plan
#define p_fftw_execute fftw_execute
#endif

#define hardscale2 0
#define EXPANSION 0
#define withCorr 1
#define withBins 1
#define LAMBDA_MODE 1
#ifndef PHN_REF_WITHCHARGE
#define PHN_REF_WITHCHARGE 0
#endif
#define withcharge PHN_REF_WITHCHARGE
#ifndef PHN_REF_EXPANSION
#define PHN_REF_EXPANSION 0
#endif
#define expansion PHN_REF_EXPANSION
#define finebin 0
#ifndef PHN_REF_ENERGYPS
#define PHN_REF_ENERGYPS 0
#endif
#define withEnergyPS PHN_REF_ENERGYPS
#define islanddetect 1
#ifndef PHN_REF_ENERGYID
#define PHN_REF_ENERGYID 0
#endif
#define EnergybasedID PHN_REF_ENERGYID
#define theory PHN_REF_THEORY
#define adjustDT 0
#ifndef PHN_REF_INIT
#define PHN_REF_INIT 3
#endif
#define initialize PHN_REF_INIT

int runs = 1;
int runID = 1;
int nodes = 1;
int ID = 0;

int Nc = 1;
int Mass_Mode = 1;
pseudo_double M_sqr = 1.;
int Lambda_Mode = -1;
pseudo_double Lambda = 1.;
pseudo_double Kappa = 2.;
pseudo_double h = 0.;
/* expanding box (parameters.cpp:177): H_0 */
pseudo_double H_0 = 0.0171156;
/* theories 2-5 (parameters.cpp:122-170) */
pseudo_double F_SSB = 1.;
pseudo_double alpha = 0.;
pseudo_double M_mono_sqr = 1.;
pseudo_double g = 2.;
pseudo_double p_mono = -0.5;

int renorm_tadpole = 0;
int max_renSteps = 2000;
pseudo_double tad_precision = 1e-6;

pseudo_double a_t = 0.25;
int N_t = 8;
pseudo_double a_eta;
int N_eta;
pseudo_double T0 = 0;
pseudo_double TMax = 1e30;
pseudo_double TSO = 1.0;
pseudo_double TMO = 1e30;
pseudo_double dtBaseTrans = 0.08;
pseudo_double dtBaseLong = 0.08;

int justnoise = 0;
pseudo_double QS = 1.;
pseudo_double scale2 = 1.;
pseudo_double Amplitude = 0.;
pseudo_double chi = 1.;
pseudo_double Noise = 0.5;
pseudo_double phi0_0 = 0., phi0_1 = 0.;
pseudo_double pi0_0 = 0., pi0_1 = 0.;
pseudo_double M2_long = 0., M2_trans = 0.;
/* initialize 0-2 (parameters.cpp:207-272): the homogeneous values phi0, pi0
 * of component 0, FAmp and Temperature (initialize 0; Temperature also in
 * initialize 4, which parameters.cpp gives no block of its own) */
pseudo_double phi0 = 0., pi0 = 0.;
pseudo_double FAmp = 0.5;
pseudo_double Temperature = 1.;

int LASTRUN = 0;

#endif

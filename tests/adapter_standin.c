/*
 * CPU stand-in for libphinum_gpu, for running the reference-side adapter
 * (phinum_gb300/adapter/phinum_dynamics.cpp) without a GPU.
 *
 * TEST INFRASTRUCTURE ONLY (tests/test_adapter.py): the entry points of
 * include/phinum_gpu.h that the adapter's run loop calls -- create, upload,
 * download, reset, evolve, the clock, averages, spectrum, islands -- are
 * implemented on the CPU oracle (oracle/phinum_oracle.c, the reference's
 * arithmetic in its own order), so a run through the adapter must write the
 * same SO and Distrib files, byte for byte, as the reference's own loop.  The
 * island tracker (Full_Analysis with history) is not provided here.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "phinum_gpu.h"
#include "phinum_oracle.h"

struct phn_handle {
  phn_params p;
  orc_params op;
  orc_clock clock;
  double *Phi, *Pi; /* reference layout, ghosts included */
  long len;
};

static char g_err[256] = "";

static int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

const char *phn_last_error(void) { return g_err; }

int phn_create(const phn_params *p, phn_handle **out) {
  if (!p || !out) return fail(PHN_ERR_INVALID, "NULL argument");
  if (p->N < 2 || p->Nc < 1 || p->Nc > PHN_MAX_NC) return fail(PHN_ERR_INVALID, "bad lattice");
  phn_handle *h = (phn_handle *)calloc(1, sizeof(phn_handle));
  h->p = *p;
  h->op.N = p->N;
  h->op.Nc = p->Nc;
  h->op.theory = p->potential;
  h->op.mass_mode = p->mass_mode;
  h->op.lambda_mode = p->lambda_mode;
  h->op.expansion = p->expanding;
  h->op.a = p->a;
  h->op.dt = p->dt;
  h->op.T0 = p->T0;
  h->op.m_sqr = p->m_sqr;
  h->op.kappa = p->kappa;
  h->op.h = p->h;
  h->op.g = p->g;
  h->op.p_mono = p->p_mono;
  h->op.m_mono_sqr = p->m_mono_sqr;
  h->op.H0 = p->H0;
  h->len = (long)p->Nc * p->N * p->N * (p->N + 2);
  h->Phi = (double *)calloc((size_t)h->len, sizeof(double));
  h->Pi = (double *)calloc((size_t)h->len, sizeof(double));
  orc_reset(&h->op, &h->clock);
  *out = h;
  return PHN_OK;
}

int phn_destroy(phn_handle *h) {
  if (!h) return PHN_OK;
  free(h->Phi);
  free(h->Pi);
  free(h);
  return PHN_OK;
}

int phn_upload(phn_handle *h, const double *Phi, const double *Pi) {
  if (!h || !Phi || !Pi) return fail(PHN_ERR_INVALID, "NULL argument");
  memcpy(h->Phi, Phi, (size_t)h->len * sizeof(double));
  memcpy(h->Pi, Pi, (size_t)h->len * sizeof(double));
  orc_exchange(&h->op, h->Phi);
  return PHN_OK;
}

int phn_download(phn_handle *h, double *Phi, double *Pi) {
  if (!h || (!Phi && !Pi)) return fail(PHN_ERR_INVALID, "NULL argument");
  const long slab = (long)h->p.Nc * h->p.N * h->p.N;
  if (Phi) memcpy(Phi, h->Phi, (size_t)h->len * sizeof(double));
  if (Pi) memcpy(Pi + slab, h->Pi + slab, (size_t)(h->len - 2 * slab) * sizeof(double));
  return PHN_OK;
}

int phn_upload_f32(phn_handle *h, const float *Phi, const float *Pi) {
  if (!h || !Phi || !Pi) return fail(PHN_ERR_INVALID, "NULL argument");
  for (long k = 0; k < h->len; k++) {
    h->Phi[k] = Phi[k];
    h->Pi[k] = Pi[k];
  }
  orc_exchange(&h->op, h->Phi);
  return PHN_OK;
}

int phn_download_f32(phn_handle *h, float *Phi, float *Pi) {
  if (!h || (!Phi && !Pi)) return fail(PHN_ERR_INVALID, "NULL argument");
  const long slab = (long)h->p.Nc * h->p.N * h->p.N;
  for (long k = 0; k < h->len; k++) {
    if (Phi) Phi[k] = (float)h->Phi[k];
    if (Pi && k >= slab && k < h->len - slab) Pi[k] = (float)h->Pi[k];
  }
  return PHN_OK;
}

int phn_reset(phn_handle *h) {
  if (!h) return fail(PHN_ERR_INVALID, "NULL handle");
  orc_reset(&h->op, &h->clock);
  return PHN_OK;
}

int phn_evolve(phn_handle *h, int nsteps) {
  if (!h || nsteps < 0) return fail(PHN_ERR_INVALID, "bad argument");
  orc_evolve(&h->op, &h->clock, h->Phi, h->Pi, nsteps, 1);
  return PHN_OK;
}

int phn_time(const phn_handle *h, double *tau, int *steps) {
  if (!h) return fail(PHN_ERR_INVALID, "NULL handle");
  if (tau) *tau = h->clock.tau;
  if (steps) *steps = h->clock.steps;
  return PHN_OK;
}

int phn_conformal_time(const phn_handle *h, double *tau_c, double *sf) {
  if (!h) return fail(PHN_ERR_INVALID, "NULL handle");
  if (tau_c) *tau_c = h->clock.tau_c;
  if (sf) *sf = h->clock.sf;
  return PHN_OK;
}

int phn_volume_averages(phn_handle *h, phn_averages *out) {
  if (!h || !out) return fail(PHN_ERR_INVALID, "NULL argument");
  orc_row r;
  orc_averages(&h->op, &h->clock, h->Phi, h->Pi, &r);
  memset(out, 0, sizeof(*out));
  out->t = h->clock.tau;
  for (int a = 0; a < PHN_MAX_NC; a++) {
    out->phi[a] = r.phi[a];
    out->pi[a] = r.pi[a];
  }
  out->phi2 = r.phi2;
  out->pi2 = r.pi2;
  out->phipi = r.phipi;
  out->phi4 = r.phi4;
  out->phi6 = r.phi6;
  out->energy = r.energy;
  out->interaction = r.interaction;
  out->charge = r.charge;
  out->min_phi = r.min_phi;
  out->max_phi = r.max_phi;
  out->max_abs_phi = r.max_abs_phi;
  out->min_pos = r.min_pos;
  out->max_pos = r.max_pos;
  out->max_abs_pos = r.max_abs_pos;
  out->gradient = r.gradient;
  out->scale_factor = h->clock.sf;
  const long slab = (long)h->p.Nc * h->p.N * h->p.N;
  for (long k = slab; k < h->len - slab; k++)
    if (!isfinite(h->Phi[k]) || !isfinite(h->Pi[k])) out->nonfinite += 1;
  return out->nonfinite > 0 ? fail(PHN_ERR_NONFINITE, "non-finite field values") : PHN_OK;
}

int phn_spectrum_bins(const phn_handle *h, int *nbins, double *binsize) {
  if (!h || !nbins || !binsize) return fail(PHN_ERR_INVALID, "NULL argument");
  orc_spectrum_bins(&h->op, nbins, binsize);
  return PHN_OK;
}

int phn_spectrum(phn_handle *h, double *F, double *K, double *Q, int *counts, int nbins) {
  int nb;
  double bs;
  if (!h || !F || !K || !Q || !counts) return fail(PHN_ERR_INVALID, "NULL argument");
  orc_spectrum_bins(&h->op, &nb, &bs);
  if (nbins < nb) return fail(PHN_ERR_TRUNCATED, "nbins %d < %d", nbins, nb);
  return orc_spectrum(&h->op, h->Phi, h->Pi, F, K, Q, counts) >= 0 ? PHN_OK : fail(PHN_ERR_INVALID, "spectrum");
}

int phn_islands(phn_handle *h, double thres, int mode, int z_periodic, int *labels, phn_island *out, int max_out,
                int *n_islands) {
  if (!h || !n_islands) return fail(PHN_ERR_INVALID, "NULL argument");
  if (h->p.Nc != 1) return fail(PHN_ERR_UNSUPPORTED, "islands need Nc = 1");
  orc_island *tmp = (orc_island *)malloc(sizeof(orc_island) * (size_t)(max_out > 0 ? max_out : 1));
  const int n = orc_islands_at(&h->op, &h->clock, h->Phi, h->Pi, thres, mode, z_periodic, labels, tmp,
                               max_out > 0 ? max_out : 0);
  for (int i = 0; i < n && i < max_out && out; i++) memcpy(&out[i], &tmp[i], sizeof(phn_island));
  free(tmp);
  *n_islands = n;
  return PHN_OK;
}

/* The tracker is not provided by this stand-in. */
int phn_tracker_create(int rank, phn_tracker **out) {
  (void)rank;
  if (out) *out = NULL;
  return fail(PHN_ERR_UNSUPPORTED, "no island tracker in the CPU stand-in");
}
int phn_tracker_update(phn_tracker *t, phn_handle *h, double thres, int mode, int z_periodic, int *labels) {
  (void)t; (void)h; (void)thres; (void)mode; (void)z_periodic; (void)labels;
  return fail(PHN_ERR_UNSUPPORTED, "no island tracker in the CPU stand-in");
}
int phn_tracker_count(const phn_tracker *t, int set, int *n) {
  (void)t; (void)set;
  if (n) *n = 0;
  return fail(PHN_ERR_UNSUPPORTED, "no island tracker in the CPU stand-in");
}
int phn_tracker_get(const phn_tracker *t, int set, int i, phn_track_island *out) {
  (void)t; (void)set; (void)i; (void)out;
  return fail(PHN_ERR_UNSUPPORTED, "no island tracker in the CPU stand-in");
}

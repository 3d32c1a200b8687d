// Island tracking over a run: Full_Analysis() with its history
// (islands.cpp:61-70, 651-840) and the consumers of the tracked islands
// (Oscillon_specific_observables, islands.cpp:745-775; add_stat_new,
// statistics.cpp:43-67).
//
// The labelling itself is the GPU union-find of islands.cu; what remains is
// host bookkeeping over one record per island, in the reference's order of
// operations:
//   1. sort found_islands by last volume, descending -- std::sort with the
//      reference's comparison (islands.cpp:30-33), so ties come out in the
//      same order as the reference's own std::sort of the same sequence;
//   2. Old_islands: islands whose centre is no longer in the mask retire;
//   3. in sorted order, an island whose centre lies in an island claimed
//      earlier in this update is merged away; otherwise it claims that island
//      and appends its statistics (BFS from the centre, islands.cpp:90-279,
//      which also resets status to 0), then the bubble and oscillon checks;
//   4. islands nobody claimed become new ones in the scan order of
//      islands.cpp:830-837 (smallest site index first).
// The centre of an entry is the island's maximum of phi^2; the reference
// takes the first maximum in BFS order, the GPU the smallest index among
// maxima -- the same site unless two sites tie exactly.
#include <math.h>

#include <algorithm>
#include <vector>

#include "phn_internal.h"

namespace phn {

struct TrackEntry {
  double at_time, center, V, pot, kin, grad, avphi, peak;
};

struct TrackIsland {
  int index, status, disp;
  int cc;  // island holding the centre in the current update
  std::vector<TrackEntry> hist;
};

}  // namespace phn

using namespace phn;

struct phn_tracker {
  int rank;
  int number_of_islands;
  std::vector<TrackIsland> alive, retired, bubbles;
  std::vector<phn_island> comps;
  std::vector<long long> centers;
  std::vector<int> cc, owner;
};

namespace phn {

static bool is_bubble(const TrackIsland &B) {  // islands.cpp:61-65
  return B.hist.back().grad + B.hist.back().pot < 0.;
}

static bool is_oscillon(const TrackIsland &B) {  // islands.cpp:67-70
  return B.hist.back().at_time - B.hist.front().at_time > 40.;
}

// One BFS result appended to an island's history (islands.cpp:243-276).
static void append(TrackIsland &B, const phn_island &c, double tau) {
  TrackEntry e;
  e.at_time = tau;
  e.center = c.peak_pos;
  e.V = c.volume;
  e.pot = c.pot_en;
  e.kin = c.kin_en;
  e.grad = c.grad_en;
  e.avphi = c.av_phi;
  e.peak = c.peak_value;
  B.hist.push_back(e);
  B.status = 0;
  if (B.hist.size() > 5) B.hist.erase(B.hist.begin() + 2);
}

static void to_record(const TrackIsland &B, phn_track_island *o) {
  o->index = B.index;
  o->status = B.status;
  o->disp = B.disp;
  o->length = (double)B.hist.size();
  for (int j = 0; j < PHN_TRACK_HISTORY; ++j) {
    const bool have = j < (int)B.hist.size();
    const TrackEntry e = have ? B.hist[(size_t)j] : TrackEntry{0, 0, 0, 0, 0, 0, 0, 0};
    o->at_time[j] = e.at_time;
    o->center[j] = e.center;
    o->volume[j] = e.V;
    o->pot_en[j] = e.pot;
    o->kin_en[j] = e.kin;
    o->grad_en[j] = e.grad;
    o->av_phi[j] = e.avphi;
    o->peak_value[j] = e.peak;
  }
}

static const std::vector<TrackIsland> *track_set(const phn_tracker *t, int set) {
  if (set == PHN_TRACK_ALIVE) return &t->alive;
  if (set == PHN_TRACK_RETIRED) return &t->retired;
  if (set == PHN_TRACK_BUBBLES) return &t->bubbles;
  return nullptr;
}

}  // namespace phn

extern "C" {

int phn_tracker_create(int rank, phn_tracker **out) {
  if (!out || rank < 0) return set_error(PHN_ERR_INVALID, "bad argument");
  phn_tracker *t = new phn_tracker();
  t->rank = rank;
  t->number_of_islands = 0;
  *out = t;
  return PHN_OK;
}

int phn_tracker_destroy(phn_tracker *t) {
  delete t;
  return PHN_OK;
}

int phn_tracker_reset(phn_tracker *t) {
  if (!t) return set_error(PHN_ERR_INVALID, "tracker is NULL");
  t->alive.clear();
  t->retired.clear();
  t->bubbles.clear();
  t->number_of_islands = 0;
  return PHN_OK;
}

int phn_tracker_update_records(phn_tracker *t, double tau, const phn_island *comps, int ncomp,
                               const int *center_island, int *owner) {
  if (!t || ncomp < 0 || (ncomp > 0 && !comps) || (!t->alive.empty() && !center_island))
    return set_error(PHN_ERR_INVALID, "bad argument");
  for (size_t i = 0; i < t->alive.size(); ++i) {
    const int c = center_island[i];
    if (c < -1 || c >= ncomp) return set_error(PHN_ERR_INVALID, "center_island[%zu] = %d", i, c);
    t->alive[i].cc = c;
  }
  t->retired.clear();
  t->bubbles.clear();
  std::vector<TrackIsland> &isl = t->alive;
  // 1. sort by last volume, descending (islands.cpp:30-33, 788)
  std::sort(isl.begin(), isl.end(),
            [](const TrackIsland &B1, const TrackIsland &B2) { return B1.hist.back().V > B2.hist.back().V; });
  // 2. Old_islands (islands.cpp:651-711)
  for (size_t i = 0; i < isl.size();) {
    if (isl[i].cc < 0) {
      t->retired.push_back(isl[i]);
      isl.erase(isl.begin() + (long)i);
    } else {
      ++i;
    }
  }
  // 3. re-seed from the centres in sorted order (islands.cpp:792-820)
  std::vector<char> claimed((size_t)ncomp, 0);
  for (size_t i = 0; i < isl.size(); ++i) {
    const int c = isl[i].cc;
    if (claimed[(size_t)c]) {  // merged into an island claimed earlier
      isl.erase(isl.begin() + (long)i);
      --i;
      continue;
    }
    claimed[(size_t)c] = 1;
    append(isl[i], comps[c], tau);
    if (is_bubble(isl[i]) && isl[i].status == 0) {
      t->bubbles.push_back(isl[i]);
      isl[i].status = 1;
    }
    if (is_oscillon(isl[i]) && isl[i].status == 0) isl[i].status = 2;
  }
  // 4. new islands in scan order (islands.cpp:822-829)
  for (int c = 0; c < ncomp; ++c) {
    if (claimed[(size_t)c]) continue;
    TrackIsland B;
    B.index = t->number_of_islands + t->rank * 1000000;
    B.disp = 1;
    B.status = 0;
    B.cc = c;
    append(B, comps[c], tau);
    t->number_of_islands++;
    isl.push_back(B);
  }
  if (owner) {
    for (int c = 0; c < ncomp; ++c) owner[c] = -1;
    for (size_t i = 0; i < isl.size(); ++i) owner[isl[i].cc] = (int)i;
  }
  return PHN_OK;
}

int phn_tracker_centers(const phn_tracker *t, long long *pos, int max, int *n) {
  if (!t || !n || (max > 0 && !pos)) return set_error(PHN_ERR_INVALID, "bad argument");
  *n = (int)t->alive.size();
  for (int i = 0; i < *n && i < max; ++i) pos[i] = (long long)t->alive[(size_t)i].hist.back().center;
  return *n > max ? set_error(PHN_ERR_TRUNCATED, "%d centres, room for %d", *n, max) : PHN_OK;
}

int phn_tracker_update(phn_tracker *t, phn_handle *h, double thres, int mode, int z_periodic, int *labels) {
  if (!t || !h) return set_error(PHN_ERR_INVALID, "NULL argument");
  // this update's islands (one labelling pass; the record buffer grows once)
  int n = 0;
  if (t->comps.empty()) t->comps.resize(1024);
  int r = phn_islands(h, thres, mode, z_periodic, nullptr, t->comps.data(), (int)t->comps.size(), &n);
  if (r == PHN_ERR_TRUNCATED) {
    t->comps.resize((size_t)n + (size_t)n / 4 + 64);
    r = phn_islands(h, thres, mode, z_periodic, nullptr, t->comps.data(), (int)t->comps.size(), &n);
  }
  if (r) return r;
  // where the alive islands' centres are now
  const int k = (int)t->alive.size();
  t->centers.resize((size_t)k);
  t->cc.resize((size_t)k);
  for (int i = 0; i < k; ++i) t->centers[(size_t)i] = (long long)t->alive[(size_t)i].hist.back().center;
  if (k > 0) {
    r = phn_islands_lookup(h, t->centers.data(), k, t->cc.data());
    if (r) return r;
  }
  double tau = 0.0;
  int steps = 0;
  r = phn_time(h, &tau, &steps);
  if (r) return r;
  t->owner.resize((size_t)(n > 0 ? n : 1));
  r = phn_tracker_update_records(t, tau, t->comps.data(), n, t->cc.data(), t->owner.data());
  if (r) return r;
  if (labels) return islands_labels_mapped(h, t->owner.data(), n, labels);
  return PHN_OK;
}

int phn_tracker_count(const phn_tracker *t, int set, int *n) {
  if (!t || !n) return set_error(PHN_ERR_INVALID, "NULL argument");
  const std::vector<TrackIsland> *v = track_set(t, set);
  if (!v) return set_error(PHN_ERR_INVALID, "set %d", set);
  *n = (int)v->size();
  return PHN_OK;
}

int phn_tracker_get(const phn_tracker *t, int set, int i, phn_track_island *out) {
  if (!t || !out) return set_error(PHN_ERR_INVALID, "NULL argument");
  const std::vector<TrackIsland> *v = track_set(t, set);
  if (!v) return set_error(PHN_ERR_INVALID, "set %d", set);
  if (i < 0 || i >= (int)v->size()) return set_error(PHN_ERR_INVALID, "island %d of %zu", i, v->size());
  to_record((*v)[(size_t)i], out);
  return PHN_OK;
}

int phn_tracker_oscillons(const phn_tracker *t, int N, double a, double avg_energy, double out[3]) {
  if (!t || !out) return set_error(PHN_ERR_INVALID, "NULL argument");
  double r_osc = 0, n_osc = 0, avgM_osc = 0.;
  for (const TrackIsland &B : t->alive)
    if (B.disp && is_oscillon(B)) {
      r_osc += (B.hist.back().pot + B.hist.back().kin + B.hist.back().grad);
      n_osc = n_osc + 1.;
    }
  avgM_osc = r_osc / n_osc;
  r_osc = r_osc / N / a / N / a / N / a / avg_energy;
  n_osc = n_osc / N / a / N / a / N / a;
  out[0] = r_osc;
  out[1] = n_osc;
  out[2] = avgM_osc;
  return PHN_OK;
}

int phn_tracker_add_stat(const phn_tracker *t, double thres, double QS, int *hist_r, int *hist_r0) {
  if (!t || !hist_r || !hist_r0) return set_error(PHN_ERR_INVALID, "NULL argument");
  const int nb = 200;  // nnnnn (statistics.cpp:17)
  for (const TrackIsland &B : t->alive) {
    if (!B.disp) continue;
    const double f = fabs(B.hist.back().peak);
    const double rr = pow(B.hist.back().V * 3. / 4. / acos(-1.), 1. / 3.);
    const double rr0 = pow(B.hist.back().V * 3. / 4. / acos(-1.), 1. / 3.) / sqrt(log(f * f / thres / thres));
    if ((f < 5 * thres) && (rr < 5. / QS)) hist_r[(int)(f / 5 / thres * nb) * nb + (int)(rr / 5. * QS * nb)]++;
    if ((f < 5 * thres) && (rr0 < 5. / QS)) hist_r0[(int)(f / 5 / thres * nb) * nb + (int)(rr0 / 5. * QS * nb)]++;
  }
  return PHN_OK;
}

}  // extern "C"

// Field checkpoints in the reference's text format: SaveConfig and
// ExtractConfig (fieldanalysis.cpp:252-312).
//
// field-<name>-<rank>.out holds one line per interior site in the reference
// layout's order (pos(0,0,1) up to the last interior index): "%.17e %.17e\n"
// of Phi and Pi from the double-precision build, "%.9e %.9e\n" from the
// single-precision one; moment-<name>.out holds tau as an ostream writes it.
// Lines are formatted by the C library's own snprintf, in parallel on host
// threads over contiguous site ranges and written in order, so the bytes are
// those the reference's fprintf loop writes; reading splits the file at line
// boundaries and parses the ranges in parallel with strtod.
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "phn_internal.h"

namespace phn {

static int io_threads(int nthreads) {
  if (nthreads > 0) return nthreads;
  const unsigned hc = std::thread::hardware_concurrency();
  return hc > 0 ? (int)hc : 1;
}

static std::string join_path(const char *dir, const std::string &file) {
  std::string d = dir && dir[0] ? dir : ".";
  if (d.back() != '/') d += '/';
  return d + file;
}

}  // namespace phn

using namespace phn;

extern "C" {

int phn_write_config_file(const char *path, const double *Phi, const double *Pi, int N, int Nc, int precision,
                          int nthreads) {
  if (!path || !Phi || !Pi || N < 1 || Nc < 1) return set_error(PHN_ERR_INVALID, "bad argument");
  FILE *of = fopen(path, "w");
  if (!of) return set_error(PHN_ERR_INVALID, "cannot open %s: %s", path, strerror(errno));
  const long long begin = (long long)Nc * N * N, end = (long long)Nc * N * N * (N + 1);
  const char *fmt = precision == PHN_FP32 ? "%.9e %.9e\n" : "%.17e %.17e\n";
  const bool single = precision == PHN_FP32;
  const int nt = io_threads(nthreads);
  // batches of nt ranges, each range formatted into its own buffer
  const long long per = 1 << 18;  // lines per range
  std::vector<std::string> buf((size_t)nt);
  int status = PHN_OK;
  for (long long b0 = begin; b0 < end && status == PHN_OK; b0 += per * nt) {
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
      const long long k0 = b0 + per * t, k1 = k0 + per < end ? k0 + per : end;
      buf[(size_t)t].clear();
      if (k0 >= end) continue;
      th.emplace_back([&, t, k0, k1]() {
        std::string &s = buf[(size_t)t];
        s.reserve((size_t)(k1 - k0) * 50);
        char line[128];
        for (long long k = k0; k < k1; ++k) {
          // the single-precision build passes floats, promoted to double
          const double a = single ? (double)(float)Phi[k] : Phi[k];
          const double c = single ? (double)(float)Pi[k] : Pi[k];
          const int n = snprintf(line, sizeof line, fmt, a, c);
          s.append(line, (size_t)n);
        }
      });
    }
    for (std::thread &x : th) x.join();
    for (int t = 0; t < nt; ++t)
      if (!buf[(size_t)t].empty() && fwrite(buf[(size_t)t].data(), 1, buf[(size_t)t].size(), of) != buf[(size_t)t].size())
        status = set_error(PHN_ERR_INVALID, "write to %s failed", path);
  }
  if (fclose(of) != 0 && status == PHN_OK) status = set_error(PHN_ERR_INVALID, "closing %s failed", path);
  return status;
}

int phn_read_config_file(const char *path, double *Phi, double *Pi, int N, int Nc, int nthreads) {
  if (!path || !Phi || !Pi || N < 1 || Nc < 1) return set_error(PHN_ERR_INVALID, "bad argument");
  FILE *f = fopen(path, "rb");
  if (!f) return set_error(PHN_ERR_INVALID, "cannot open %s: %s", path, strerror(errno));
  std::string data;
  if (fseek(f, 0, SEEK_END) == 0) {
    const long sz = ftell(f);
    if (sz > 0) {
      data.resize((size_t)sz);
      fseek(f, 0, SEEK_SET);
      if (fread(&data[0], 1, (size_t)sz, f) != (size_t)sz) data.clear();
    }
  }
  fclose(f);
  const long long begin = (long long)Nc * N * N, lines = (long long)Nc * N * N * N;
  // line starts
  std::vector<size_t> starts;
  starts.reserve((size_t)lines + 1);
  size_t p = 0;
  while (p < data.size() && (long long)starts.size() < lines) {
    starts.push_back(p);
    const void *nl = memchr(data.data() + p, '\n', data.size() - p);
    if (!nl) break;
    p = (size_t)((const char *)nl - data.data()) + 1;
  }
  if ((long long)starts.size() < lines)
    return set_error(PHN_ERR_INVALID, "%s: %zu lines, %lld expected", path, starts.size(), lines);
  const int nt = io_threads(nthreads);
  std::vector<int> bad((size_t)nt, 0);
  std::vector<std::thread> th;
  const long long per = (lines + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const long long l0 = per * t, l1 = l0 + per < lines ? l0 + per : lines;
    if (l0 >= l1) continue;
    th.emplace_back([&, t, l0, l1]() {
      for (long long l = l0; l < l1; ++l) {
        const char *s = data.c_str() + starts[(size_t)l];
        char *e1 = nullptr, *e2 = nullptr;
        const double a = strtod(s, &e1);
        const double c = strtod(e1, &e2);
        if (e1 == s || e2 == e1) {
          bad[(size_t)t] = 1;
          return;
        }
        Phi[begin + l] = a;
        Pi[begin + l] = c;
      }
    });
  }
  for (std::thread &x : th) x.join();
  for (int b : bad)
    if (b) return set_error(PHN_ERR_INVALID, "%s: malformed line", path);
  return PHN_OK;
}

int phn_save_config(phn_handle *h, const char *dir, int name, int rank, int nthreads) {
  if (!h || rank < 0) return set_error(PHN_ERR_INVALID, "bad argument");
  const size_t n = (size_t)h->p.Nc * h->p.N * h->p.N * (h->p.N + 2);
  std::vector<double> phi(n), pi(n, 0.0);
  int r = phn_download(h, phi.data(), pi.data());
  if (r) return r;
  char file[96];
  snprintf(file, sizeof file, "field-%i-%i.out", name, rank);
  r = phn_write_config_file(join_path(dir, file).c_str(), phi.data(), pi.data(), h->p.N, h->p.Nc, h->p.precision,
                            nthreads);
  if (r || rank != 0) return r;
  snprintf(file, sizeof file, "moment-%i.out", name);
  const std::string path = join_path(dir, file);
  FILE *mf = fopen(path.c_str(), "w");
  if (!mf) return set_error(PHN_ERR_INVALID, "cannot open %s", path.c_str());
  std::ostringstream os;  // fout << LocalLattice::tau << endl (fieldanalysis.cpp:280)
  os << h->tau << '\n';
  const std::string t = os.str();
  const bool ok = fwrite(t.data(), 1, t.size(), mf) == t.size();
  fclose(mf);
  return ok ? PHN_OK : set_error(PHN_ERR_INVALID, "write to %s failed", path.c_str());
}

int phn_load_config(phn_handle *h, const char *dir, int name, int rank, double *t0, int nthreads) {
  if (!h || rank < 0) return set_error(PHN_ERR_INVALID, "bad argument");
  const size_t n = (size_t)h->p.Nc * h->p.N * h->p.N * (h->p.N + 2);
  std::vector<double> phi(n, 0.0), pi(n, 0.0);
  char file[96];
  snprintf(file, sizeof file, "field-%i-%i.out", name, rank);
  int r = phn_read_config_file(join_path(dir, file).c_str(), phi.data(), pi.data(), h->p.N, h->p.Nc, nthreads);
  if (r) return r;
  r = phn_upload(h, phi.data(), pi.data());
  if (r) return r;
  if (t0) {
    snprintf(file, sizeof file, "moment-%i.out", name);
    const std::string path = join_path(dir, file);
    FILE *mf = fopen(path.c_str(), "r");
    if (!mf) return set_error(PHN_ERR_INVALID, "cannot open %s", path.c_str());
    double v = 0.0;
    const int got = fscanf(mf, "%lf", &v);
    fclose(mf);
    if (got != 1) return set_error(PHN_ERR_INVALID, "%s: no time stamp", path.c_str());
    *t0 = v;
  }
  return PHN_OK;
}

}  // extern "C"

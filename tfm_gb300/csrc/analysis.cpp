// Statistics and writers of ccp-analyze's outputs (see analysis.h).
#include "analysis.h"

#include <cmath>
#include <cstdio>
#include <cstring>

#include "host.h"

namespace ccpgpu {

Stat stats_plain(const std::vector<float> &v) {
  // float values and their float squares, summed in double in order
  double m1 = 0.0, m2 = 0.0;
  const size_t n = v.size();
  for (float x : v) {
    m1 += x;
    m2 += x * x;
  }
  m1 /= (double)n;
  m2 /= (double)n;
  Stat s;
  s.avg = m1;
  s.var = (m2 - m1 * m1) / (1.0 - 1.0 / (double)n);
  s.sem = std::sqrt(s.var / (double)n);
  return s;
}

void stats_blocked(const std::vector<float> &v, Stat &s, uint32_t &n_blocks) {
  std::vector<float> av = v;
  Stat p = stats_plain(av);
  s = p;
  size_t n = av.size();
  double ivm = p.var / (double)n;
  double ul = ivm * (1.0 + std::sqrt(2.0 / ((double)n - 1.0)));
  // a series too short to block keeps the unblocked error
  s.sem = std::sqrt(ivm);
  n_blocks = (uint32_t)n;
  while (n >= 4) {
    size_t b = 0;
    for (; 2 * b + 1 < n; ++b) av[b] = 0.5 * (av[2 * b] + av[2 * b + 1]);
    n = b;
    av.resize(n);
    Stat q = stats_plain(av);
    ivm = q.var / (double)n;
    s.sem = std::sqrt(ivm);
    n_blocks = (uint32_t)n;
    if (ivm > ul)
      ul = ivm * (1.0 + std::sqrt(2.0 / ((double)n - 1.0)));
    else
      break;
  }
}

SeriesStat stats_series(const std::vector<float> &v) {
  const size_t n0 = v.size();
  double best = INFINITY;
  size_t it = n0 / 2;
  for (size_t d = 2; d < 128; d *= 2) {
    const size_t i_t = n0 / d;
    std::vector<float> av(v.begin() + i_t, v.end());
    const size_t ne = av.size();
    const Stat p = stats_plain(av);
    const double mse = p.var * (double)(ne - 1) / (double)(ne * ne);
    if (mse < best) {
      best = mse;
      it = i_t;
    }
  }
  SeriesStat r;
  r.i_t = (uint32_t)it;
  r.thermalised = it != n0 / 2;
  Stat s;
  uint32_t nb = 0;
  stats_blocked(std::vector<float>(v.begin() + it, v.end()), s, nb);
  r.avg = s.avg;
  r.var = s.var;
  r.sem = s.sem;
  r.n_blocks = nb;
  return r;
}

void SeriesCombine::add(const SeriesStat &s) {
  double w = 1.0 / (s.sem * s.sem);
  if (!std::isfinite(w)) w = 1.0;
  m1 += w * s.avg;
  m2 += w * s.avg * s.avg;
  w1 += w;
  w2 += w * w;
}

Stat SeriesCombine::result() const {
  const double a = m1 / w1, b = m2 / w1;
  Stat s;
  s.avg = a;
  s.var = (b - a * a) / (1.0 - w2 / (w1 * w1));
  s.sem = std::sqrt(s.var * w2 / (w1 * w1));
  return s;
}

void BasicCombine::add(double a) {
  m1 += a;
  m2 += a * a;
  ++n;
}

Stat BasicCombine::result() const {
  const double a = m1 / (double)n, b = m2 / (double)n;
  Stat s;
  s.avg = a;
  s.var = (b - a * a) / (1.0 - 1.0 / (double)n);
  s.sem = std::sqrt(s.var / (double)n);
  return s;
}

// ---------------------------------------------------------------- text

// ccp's cnfs(x, 12, ' ', 6): fixed, 6 decimals, width 12 (printf's %12.6f,
// including the sign of a NaN).
static void f6(std::string &o, double x) {
  char b[64];
  std::snprintf(b, sizeof b, "%12.6f", x);
  o += b;
}

static void u8w(std::string &o, unsigned long long x) {
  char b[32];
  std::snprintf(b, sizeof b, "%8llu", x);
  o += b;
}

static void series_line(std::string &o, const SeriesStat &s) {  // sostat.cu:20-26
  f6(o, s.avg);
  f6(o, std::sqrt(s.var));
  f6(o, s.sem);
  u8w(o, s.n_blocks);
  u8w(o, s.i_t);
  o += s.thermalised ? " yes\n" : "  no\n";
}

static void stat_line(std::string &o, double avg, double var, double sem) {  // sostat.cu:28-41
  f6(o, avg);
  f6(o, std::sqrt(var));
  f6(o, sem);
  o += "\n";
}

static double shell_radius(float R_n, int b) {
  return (double)R_n * std::pow((b + 1.0) / ANA_SHELLS, 1.0 / 3);
}

static void sep_index(std::string &o, int s) {
  char b[16];
  std::snprintf(b, sizeof b, "%6d", s);
  o += b;
}

void Analysis::resize(int n_systems) {
  series.assign(n_systems, std::vector<std::vector<float>>(ANA_SERIES));
  last_txt.assign(n_systems, std::string());
}

void Analysis::add_frame(int s, const float *values) {
  for (int k = 0; k < ANA_SERIES; ++k) series[s][k].push_back(values[k]);
}

void Analysis::finish(int s, const AnaLayout &lay, const std::vector<std::vector<double>> &sd,
                      const std::vector<std::vector<double>> &cp, const std::vector<double> &cm) {
  std::vector<SeriesStat> st(ANA_SERIES);
  for (int k = 0; k < ANA_SERIES; ++k) st[k] = stats_series(series[s][k]);

  // analysis-XXX.dat (chrana.cu:205-256)
  std::string o = "         avg   sqrt(var)         sem   f_n_b     i_t ter\n";
  for (int k = 0; k < 4; ++k) series_line(o, st[k]);
  o += "\n\n";
  for (int t = 0; t < 3; ++t) {
    o += "         r_b         avg   sqrt(var)         sem\n";
    o += "    0.000000    0.000000    0.000000    0.000000\n";
    for (int b = 0; b < ANA_SHELLS; ++b) {
      f6(o, shell_radius(lay.R_n, b));
      const SeriesStat &q = st[4 + t * ANA_SHELLS + b];
      stat_line(o, q.avg, q.var, q.sem);
    }
    o += "\n\n";
  }
  for (const auto *arr : {&sd, &cp}) {
    for (size_t blk = 0; blk < lay.block_len.size(); ++blk) {
      o += "     s         avg\n";
      for (int i = 0; i < lay.block_len[blk]; ++i) {
        sep_index(o, i + 1);
        f6(o, (*arr)[blk][i]);
        o += "\n";
      }
      o += "\n\n";
    }
  }
  last_txt[s] = std::move(o);

  // combination over simulations that share the layout
  if (!have_layout) {
    layout = lay;
    have_layout = true;
    comb_series.assign(ANA_SERIES, SeriesCombine());
    comb_sd.assign(lay.block_len.size(), {});
    comb_cp.assign(lay.block_len.size(), {});
    for (size_t blk = 0; blk < lay.block_len.size(); ++blk) {
      comb_sd[blk].assign(lay.block_len[blk], BasicCombine());
      comb_cp[blk].assign(lay.block_len[blk], BasicCombine());
    }
    cm_m1.assign(lay.cm_len, 0.0);
    cm_m2.assign(lay.cm_len, 0.0);
  }
  if (!(lay == layout)) {
    mixed = true;
  } else {
    for (int k = 0; k < ANA_SERIES; ++k) comb_series[k].add(st[k]);
    for (size_t blk = 0; blk < lay.block_len.size(); ++blk)
      for (int i = 0; i < lay.block_len[blk]; ++i) {
        comb_sd[blk][i].add(sd[blk][i]);
        comb_cp[blk][i].add(cp[blk][i]);
      }
    for (int64_t k = 0; k < lay.cm_len; ++k) {
      cm_m1[k] += cm[k];
      cm_m2[k] += cm[k] * cm[k];
    }
    ++simulations;
  }
  for (auto &v : series[s]) v.clear();
}

std::string Analysis::final_txt() const {
  if (!simulations) throw Error(ST_STATE, "no finished analysis simulation");
  if (mixed) throw Error(ST_STATE, "analysed systems differ in size or radius: no combined statistics");
  // analysis-fin.dat (chrana.cu:306-360)
  std::string o = "         avg   sqrt(var)         sem\n";
  for (int k = 0; k < 4; ++k) {
    const Stat s = comb_series[k].result();
    stat_line(o, s.avg, s.var, s.sem);
  }
  o += "\n\n";
  for (int t = 0; t < 3; ++t) {
    o += "         r_b         avg   sqrt(var)         sem\n";
    o += "    0.000000    0.000000    0.000000    0.000000\n";
    for (int b = 0; b < ANA_SHELLS; ++b) {
      f6(o, shell_radius(layout.R_n, b));
      const Stat s = comb_series[4 + t * ANA_SHELLS + b].result();
      stat_line(o, s.avg, s.var, s.sem);
    }
    o += "\n\n";
  }
  for (const auto *comb : {&comb_sd, &comb_cp}) {
    for (size_t blk = 0; blk < layout.block_len.size(); ++blk) {
      o += "     s         avg   sqrt(var)         sem\n";
      for (int i = 0; i < layout.block_len[blk]; ++i) {
        sep_index(o, i + 1);
        const Stat s = (*comb)[blk][i].result();
        stat_line(o, s.avg, s.var, s.sem);
      }
      o += "\n\n";
    }
  }
  return o;
}

std::string Analysis::contact_map_bin() const {
  if (!simulations) throw Error(ST_STATE, "no finished analysis simulation");
  if (mixed) throw Error(ST_STATE, "analysed systems differ in size or radius: no combined statistics");
  std::string o(sizeof(double) * (size_t)layout.cm_len, '\0');
  for (int64_t k = 0; k < layout.cm_len; ++k) {
    const double a = cm_m1[k] / (double)simulations;  // the combined average (sostat.cu:206-224)
    std::memcpy(&o[sizeof(double) * (size_t)k], &a, sizeof(double));
  }
  return o;
}

}  // namespace ccpgpu

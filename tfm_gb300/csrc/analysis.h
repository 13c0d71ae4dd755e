// ccp-analyze's outputs fed by the engine's GPU observables: per-frame time
// series, their statistics (Program/src/sostat.cu:68-237) and the three
// files ccp-analyze writes, analysis-XXX.dat, analysis-fin.dat and
// contact-map.bin (Program/src/chrana.cu:205-369). Plain C++.
//
// A "simulation" is one run of one system between two ends of analysis
// (ccp-analyze: one initial condition and its trajectory files). In a batch
// every system is a simulation of its own; the final statistics combine all
// simulations finished so far.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace ccpgpu {

constexpr int ANA_SHELLS = 64;              // radial bins (chrana.cuh:16)
constexpr int ANA_SERIES = 4 + 3 * ANA_SHELLS;  // dcm, rg2, nop, ncf, rcd[3][64]
constexpr int ANA_MIN_BLOCKS = 6;           // sd / cp blocks ccp writes (n_chr_h)

struct Stat {
  double avg, var, sem;
};

struct SeriesStat {
  double avg, var, sem;
  uint32_t n_blocks;  // blocks left when the blocking method stopped
  uint32_t i_t;       // thermalisation index
  bool thermalised;
};

// Plain moments of single-precision values (sostat.cu:69-88).
Stat stats_plain(const std::vector<float> &v);
// Blocking method for the standard error of correlated values (sostat.cu:90-134).
void stats_blocked(const std::vector<float> &v, Stat &s, uint32_t &n_blocks);
// Marginal-standard-error thermalisation, then blocking (sostat.cu:136-174).
SeriesStat stats_series(const std::vector<float> &v);

// Inverse-variance combination of per-simulation series statistics
// (sostat.cu:176-204), accumulated one simulation at a time.
struct SeriesCombine {
  double m1 = 0, m2 = 0, w1 = 0, w2 = 0;
  void add(const SeriesStat &s);
  Stat result() const;
};

// Plain combination of per-simulation averages (sostat.cu:206-224).
struct BasicCombine {
  double m1 = 0, m2 = 0;
  uint64_t n = 0;
  void add(double a);
  Stat result() const;
};

// The shape of one system's analysis; simulations are combined only when
// their layouts agree.
struct AnaLayout {
  int n_beads = 0;
  float R_n = 0;
  std::vector<int> block_len;  // rows (separations 1, 2, ...) of each sd / cp block
  int64_t cm_len = 0;          // packed lower-triangular contact map
  bool operator==(const AnaLayout &o) const {
    return n_beads == o.n_beads && R_n == o.R_n && block_len == o.block_len && cm_len == o.cm_len;
  }
};

struct Analysis {
  // time series of the current simulation, per system: [sys][series][frame]
  std::vector<std::vector<std::vector<float>>> series;
  std::vector<std::string> last_txt;  // analysis-XXX.dat of each system's last simulation
  AnaLayout layout;
  bool have_layout = false, mixed = false;
  int64_t simulations = 0;
  std::vector<SeriesCombine> comb_series;
  std::vector<std::vector<BasicCombine>> comb_sd, comb_cp;
  std::vector<double> cm_m1, cm_m2;  // running sums of the per-simulation map averages

  void resize(int n_systems);
  // Appends one frame of system s (values: ANA_SERIES floats).
  void add_frame(int s, const float *values);
  int frames(int s) const { return series.empty() || series[s].empty() ? 0 : (int)series[s][0].size(); }
  // Ends system s's simulation: statistics of its series, its frame-averaged
  // sd / cp blocks and contact-map values; writes last_txt[s]; adds it to the
  // combination; clears the series.
  void finish(int s, const AnaLayout &lay, const std::vector<std::vector<double>> &sd,
              const std::vector<std::vector<double>> &cp, const std::vector<double> &cm);
  std::string final_txt() const;   // analysis-fin.dat
  std::string contact_map_bin() const;  // contact-map.bin: float64 averages
};

}  // namespace ccpgpu

// Host-only driver around the reference's statistics (Program/src/sostat.cu,
// compiled where it lies by oracle/ref/build_sostat.sh) that prints what
// ccp-analyze would write for given time series: per simulation the
// save_last_is_stat line of a time-series observable (sostat.cu:20-26) and
// the basic average of a basic observable (sostat.cu:47-59); then the
// combined lines (save_cs_final_stat, sostat.cu:36-41 and 61-66).
// Input (stdin): n_sims, then per simulation n_values and the values (the
// basic observable of a simulation is the plain mean of its values).
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "sostat.cuh"

int main() {
  unsigned n_sims = 0;
  if (!(std::cin >> n_sims)) return 1;
  mmc::simobs ts;
  mmc::simobs_b bs;
  std::ofstream out("/dev/stdout");
  for (unsigned s = 0; s < n_sims; ++s) {
    unsigned n = 0;
    std::cin >> n;
    ts.is_ts.clear();
    bs.is_o_sum = 0.0;
    bs.is_n_dp = 0;
    for (unsigned i = 0; i < n; ++i) {
      float v;
      std::cin >> v;
      ts.is_ts.push_back(v);
      bs.is_o_sum += v;
      ++bs.is_n_dp;
    }
    ts.calc_last_is_stat();
    bs.calc_last_is_stat();
    out << "ts ";
    ts.save_last_is_stat(out);
    out << "ts_s ";
    ts.save_last_is_stat_s(out);
    out << "b ";
    bs.save_last_is_stat(out);
  }
  ts.calc_cs_final_stat();
  bs.calc_cs_final_stat();
  out << "ts_fin ";
  ts.save_cs_final_stat(out);
  out << "b_fin ";
  bs.save_cs_final_stat(out);
  out.flush();
  return 0;
}

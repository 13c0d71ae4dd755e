// Host-only driver around the reference's own chromatin analysis
// (Program/src/chrana.cu, chrdat.cu, sostat.cu, util.cu, compiled where they
// lie by oracle/ref/build_chrana.sh and linked against the host stand-ins of
// oracle/ref/host_cuda_stub.c). TEST INFRASTRUCTURE: it prints the per-frame
// observables that chrana::calc_observables (chrana.cu:371-480) computes on
// the host, for tests/golden/make_chrana_golden.py.
//
// Usage: chrana_driver <parameter file> <initial .gro> <trajectory .trr> <out>
// The analysis reads the .gro (types and a first frame) with
// add_initial_condition and every frame of the .trr with add_trajectory_file
// (frames_per_file frames), as ccp-analyze does (ccp-analyze.cu:52-80); <out>
// gets one line per frame: t dcm rg2 nop ncf, then rcd[3][64], in %.9e.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

// the per-frame series are private members of chrana: read them directly
#define private public
#include "chrana.cuh"
#undef private

int main(int argc, char **argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: %s params.dat initial.gro trajectory.trr out.txt\n", argv[0]);
    return 2;
  }
  try {
    std::ifstream par_f(argv[1]);
    mmc::check_file(par_f, argv[1]);
    mmc::parmap par(par_f);
    mmc::chrana ana(par);
    std::ifstream gro(argv[2]);
    mmc::check_file(gro, argv[2]);
    ana.add_initial_condition(gro);
    std::ifstream trr(argv[3], std::ios::binary);
    mmc::check_file(trr, argv[3]);
    ana.add_trajectory_file(trr);
    FILE *out = std::fopen(argv[4], "w");
    if (!out) return 3;
    size_t nf = ana.t_o.is_ts.size();
    for (size_t k = 0; k < nf; ++k) {
      std::fprintf(out, "%.9e %.9e %.9e %.9e %.9e", ana.t_o.is_ts[k], ana.dcm_o.is_ts[k],
                   ana.rg2_o.is_ts[k], ana.nop_o.is_ts[k], ana.ncf_o.is_ts[k]);
      for (int t = 0; t < 3; ++t)
        for (unsigned b = 0; b < mmc::n_b; ++b)
          std::fprintf(out, " %.9e", ana.rcd_o[t][b].is_ts[k]);
      std::fprintf(out, "\n");
    }
    std::fclose(out);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "chrana_driver: %s\n", e.what());
    return 1;
  }
  return 0;
}

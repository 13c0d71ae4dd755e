"""The header-only mmc::chrsim shim compiles against a ccp-style host program
and links against libccpgpu.so (CPU only: the program is built, not run)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# a minimal stand-in for ccp's util.cuh declarations the shim relies on
UTIL = r"""
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
namespace mmc {
struct error : std::runtime_error { error(const std::string &m) : std::runtime_error(m) {} };
struct logger { static void record(const std::string &m) { std::cout << m << "\n"; } };
struct parmap : std::map<std::string, std::string> {
  parmap(std::istream &s) { std::string k, v; while (s >> k >> v) insert({k, v}); }
};
}
"""

# the calls ccp-perform.cu makes on its simulation object (ccp-perform.cu:48-111)
MAIN = r"""
#include "util_stub.h"
#include "ccpgpu_chrsim.hpp"
int main(int argc, char **argv) {
  std::ifstream inp_f(argv[1]);
  mmc::parmap par(inp_f);
  try {
    mmc::chrsim sim(par);
    sim.generate_initial_condition();
    std::ofstream out_f("initial-condition-000.gro");
    sim.write_frame_txt(out_f);
    std::ofstream lbs_f("lamina-binding-sites-000.gro");
    sim.write_lbs_txt(lbs_f);
    std::ofstream trr_f("trajectory-000-000.trr", std::ios::binary);
    sim.run_simulation(trr_f);
    std::ofstream ck_f("checkpoint-000.bin", std::ios::binary);
    sim.save_checkpoint(ck_f);
    std::ifstream ck_in("checkpoint-000.bin", std::ios::binary);
    sim.load_checkpoint(ck_in);
  } catch (const mmc::error &e) {
    std::cerr << e.what() << "\n";
    return 1;
  }
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_shim_compiles_and_links(engine_lib, tmp_path):
    (tmp_path / "util_stub.h").write_text(UTIL)
    (tmp_path / "main.cpp").write_text(MAIN)
    libdir = os.path.join(ROOT, "tfm_gb300")
    r = subprocess.run(["g++", "-std=c++17", "-I", str(tmp_path), "-I", os.path.join(ROOT, "include"),
                        str(tmp_path / "main.cpp"), "-L", libdir, "-lccpgpu",
                        "-Wl,-rpath," + libdir, "-o", str(tmp_path / "ccp-perform-gpu")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "ccp-perform-gpu").exists()

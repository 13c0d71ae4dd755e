"""The drop-in boundary for ccp's programs: the header-only mmc::chrsim shim
(include/ccpgpu_chrsim.hpp) over libccpgpu.so.

  * CPU: the reference's own ccp-perform.cu and ccp-profile.cu compile and
    link unchanged against the shim, built as a maintainer would
    (oracle/ref/build_ccp_programs.sh; skipped without a reference checkout);
  * CPU: a program making ccp-perform's calls (ccp-perform.cu:25-128) over a
    stand-in of ccp's util.cuh compiles and links;
  * GPU: that program runs a new simulation and continues it, and its files
    have ccp's layouts: the .gro initial condition and lamina sites
    (chrdat.cu:107-133, 229-254), the .trr frames (chrdat.cu:168-194) and the
    checkpoint (chrsim.cu:525-555), which the continued run reads back.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# a stand-in for the declarations of ccp's util.cuh that ccp-perform.cu and
# the shim use (util.cuh:20-113)
UTIL = r"""
#include <glob.h>
#include <iomanip>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
namespace mmc {
struct error : std::runtime_error { error(const std::string &m) : std::runtime_error(m) {} };
struct logger {
  static void set_file(const std::string &) {}
  static void record(const std::string &m) { std::cout << m << "\n"; }
};
struct parmap : std::map<std::string, std::string> {
  parmap(std::istream &s) { std::string k, v; while (s >> k >> v) insert({k, v}); }
};
template <typename T> std::string cnfs(T num, int len = 0, char fillc = ' ', int prc = 0) {
  std::stringstream s;
  if (len > 0) s << std::setw(len);
  if (fillc != ' ') s << std::setfill(fillc);
  if (prc > 0) s << std::setprecision(prc) << std::fixed;
  s << num;
  return s.str();
}
template <typename T> void check_file(T &f, const std::string &p) {
  if (!f.is_open()) throw error("unable to open " + p);
}
inline unsigned glob_count(const std::string &pat) {
  glob_t g;
  unsigned n = (glob(pat.c_str(), 0, nullptr, &g) == 0) ? (unsigned)g.gl_pathc : 0u;
  globfree(&g);
  return n;
}
}
"""

# ccp-perform's sequence of calls on its simulation object (ccp-perform.cu:25-128):
# <dir> starts simulation i_s = number of initial conditions; <dir> <i_s>
# continues it from its checkpoint into the next trajectory file
MAIN = r"""
#include "util_stub.h"
#include "ccpgpu_chrsim.hpp"
int main(int argc, char **argv) {
  const std::string dir = argv[1];
  bool new_sim = argc == 2;
  try {
    std::ifstream inp_f(dir + "/adjustable-parameters.dat");
    mmc::check_file(inp_f, dir + "/adjustable-parameters.dat");
    mmc::parmap par(inp_f);
    inp_f.close();
    mmc::chrsim sim(par);
    unsigned i_s, i_t_f;
    if (new_sim) {
      i_s = mmc::glob_count(dir + "/initial-condition-*");
      i_t_f = 0;
      sim.generate_initial_condition();
      std::ofstream out_f(dir + "/initial-condition-" + mmc::cnfs(i_s, 3, '0') + ".gro");
      sim.write_frame_txt(out_f);
      std::ofstream lbs_f(dir + "/lamina-binding-sites-" + mmc::cnfs(i_s, 3, '0') + ".gro");
      sim.write_lbs_txt(lbs_f);
    } else {
      i_s = std::stoi(argv[2]);
      i_t_f = mmc::glob_count(dir + "/trajectory-" + mmc::cnfs(i_s, 3, '0') + "*");
      std::ifstream ck(dir + "/checkpoint-" + mmc::cnfs(i_s, 3, '0') + ".bin", std::ios::binary);
      mmc::check_file(ck, "checkpoint");
      sim.load_checkpoint(ck);
    }
    std::ofstream trr_f(dir + "/trajectory-" + mmc::cnfs(i_s, 3, '0') + "-" +
                        mmc::cnfs(i_t_f, 3, '0') + ".trr", std::ios::binary);
    sim.run_simulation(trr_f);
    trr_f.close();
    std::ofstream ck_f(dir + "/checkpoint-" + mmc::cnfs(i_s, 3, '0') + ".bin", std::ios::binary);
    sim.save_checkpoint(ck_f);
  } catch (const mmc::error &e) {
    std::cerr << e.what() << "\n";
    return 1;
  }
  return 0;
}
"""


def _build_program(tmp_path):
    (tmp_path / "util_stub.h").write_text(UTIL)
    (tmp_path / "main.cpp").write_text(MAIN)
    libdir = os.path.join(ROOT, "tfm_gb300")
    exe = tmp_path / "ccp-perform-gpu"
    r = subprocess.run(["g++", "-std=c++17", "-I", str(tmp_path), "-I",
                        os.path.join(ROOT, "include"), str(tmp_path / "main.cpp"), "-L", libdir,
                        "-lccpgpu", "-Wl,-rpath," + libdir, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_ccp_programs_compile_unchanged(engine_lib):
    recipe = os.path.join(ROOT, "oracle", "ref", "build_ccp_programs.sh")
    r = subprocess.run([recipe], capture_output=True, text=True)
    if r.returncode == 3:
        pytest.skip("no reference checkout on this machine")
    assert r.returncode == 0, r.stderr[-3000:]
    out = r.stdout.strip().splitlines()[-1]
    for prog in ("ccp-perform", "ccp-profile"):
        assert os.access(os.path.join(out, prog), os.X_OK), prog


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_shim_compiles_and_links(engine_lib, tmp_path):
    assert _build_program(tmp_path).exists()


def _trr_frames(path, n):
    b = open(path, "rb").read()
    size = 72 + 12 * n
    assert len(b) % size == 0
    out = []
    for k in range(len(b) // size):
        h = np.frombuffer(b[k * size:k * size + 72], np.uint32)
        assert h[0] == 1993 and h[1] == 1 and h[10] == 12 * n and h[13] == n
        t = float(h[16:17].view(np.float32)[0])
        out.append((int(h[14]), t, np.frombuffer(b[k * size + 72:(k + 1) * size], np.float32)
                    .reshape(n, 3)))
    return out


@pytest.mark.gpu
@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_shim_program_runs_new_and_continued(engine_lib, tmp_path):
    from helpers import ccp_params

    exe = _build_program(tmp_path)
    sim_dir = tmp_path / "sim"
    sim_dir.mkdir()
    n = 256
    txt, R, n_l = ccp_params(n)
    (sim_dir / "adjustable-parameters.dat").write_text(txt + "frames_per_file 0002\nseed 7\n")
    for args in ([str(sim_dir)], [str(sim_dir), "0"]):
        r = subprocess.run([str(exe)] + args, capture_output=True, text=True, cwd=tmp_path,
                           timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
    # initial condition: "i_f t", N, one line per bead, the box line
    gro = (sim_dir / "initial-condition-000.gro").read_text().splitlines()
    assert gro[0].split() == ["0", "0"] and int(gro[1]) == n and len(gro) == n + 3
    types = [ln[5:10].strip() for ln in gro[2:2 + n]]
    assert set(types) <= {"A", "B"} and int(gro[2][:5]) == 1 and int(gro[1 + n][:5]) == n
    x0 = np.array([[float(v) for v in ln[20:44].split()] for ln in gro[2:2 + n]])
    assert (np.linalg.norm(x0, axis=1) < R).all()
    lbs = (sim_dir / "lamina-binding-sites-000.gro").read_text().splitlines()
    assert len([ln for ln in lbs if ln[5:10].strip() == "C"]) == n_l
    # two trajectory files of two frames, frame index and time continuing
    # (one time unit per frame of 2048 steps)
    f0 = _trr_frames(sim_dir / "trajectory-000-000.trr", n)
    f1 = _trr_frames(sim_dir / "trajectory-000-001.trr", n)
    assert [(i, t) for i, t, _ in f0 + f1] == [(1, 1.0), (2, 2.0), (3, 3.0), (4, 4.0)]
    for _, _, x in f0 + f1:
        assert np.isfinite(x).all() and (np.linalg.norm(x, axis=1) < R + 0.5).all()
    # checkpoint: uint32 i_f, float32 t, int32 types, float32 positions and sites
    ck = (sim_dir / "checkpoint-000.bin").read_bytes()
    assert len(ck) == 8 + 4 * n + 12 * n + 12 * n_l
    assert np.frombuffer(ck[:4], np.uint32)[0] == 4
    assert np.frombuffer(ck[4:8], np.float32)[0] == 4.0
    ptc = np.frombuffer(ck[8:8 + 4 * n], np.int32)
    assert [("A" if p == 0 else "B") for p in ptc] == types
    xk = np.frombuffer(ck[8 + 4 * n:8 + 16 * n], np.float32).reshape(n, 3)
    assert np.array_equal(xk, f1[-1][2])

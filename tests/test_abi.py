"""CPU tests of the C-ABI library: it loads, exports every symbol the header
declares, and rejects bad parameters with ccp's messages before touching the
GPU (chrdat.cu:21-63, chrsim.cu:428-435)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "ccpgpu.h")).read()
    return sorted(set(re.findall(r"\b(ccpgpu_[a-z_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(engine_lib):
    from tfm_gb300 import ccpgpu

    decl = _declared()
    assert len(decl) >= 25
    for name in decl:
        assert hasattr(engine_lib, name), name
    assert set(decl) == set(ccpgpu.SYMBOLS)


@pytest.mark.parametrize("text,msg", [
    ("number_of_particles 0\nnucleus_radius 10\n", "number_of_particles out of range"),
    ("number_of_particles 100000\nnucleus_radius 60\n", "number_of_particles out of range"),
    ("number_of_particles 1000\n", "nucleus_radius out of range"),
    ("number_of_particles 1000\nnucleus_radius 120\n", "nucleus_radius out of range"),
    ("number_of_particles 1000\nnucleus_radius 10\nopening_radius 11\n", "opening_radius out of range"),
    ("number_of_particles 1000\nnucleus_radius 10\nopening_radius 2\nbleb_radius 1\n",
     "bleb_radius out of range"),
    ("number_of_particles 1000\nnucleus_radius 10\ntemperature 2000\n", "temperature out of range"),
    ("number_of_particles 1000\nnucleus_radius 10\nframes_per_file 0\n", "frames_per_file out of range"),
    ("number_of_particles 1000\nnucleus_radius 4\n", "chromatin volume fraction above 0.4"),
    ("number_of_particles 1000\nnucleus_radius 10\nnumber_of_lbs 5000\n", "lbs area fraction above 0.4"),
    ("number_of_particles 1000\nnucleus_radius 10\nsteps_per_frame 0\n", "steps_per_frame out of range"),
    ("number_of_particles 1000\nnucleus_radius 10\nthreads_per_block 2000\n",
     "threads_per_block out of range"),
    ("force_field lj\n", "force_field out of range"),
    ("force_field baseline\nnumber_of_particles 1000\ncell_side 1.0\n",
     "cell_side below interaction cutoff"),
    ("force_field baseline\nnumber_of_particles 1000\npair_kernel 7\n", "pair_kernel out of range"),
    ("force_field baseline\nnumber_of_particles 1000\npair_lanes 3\n", "pair_lanes out of range"),
    ("force_field baseline\nnumber_of_particles 1000\nnumber_of_chains 1001\n",
     "number_of_chains out of range"),
    ("force_field baseline\nnumber_of_particles 1000\ncontact_cutoff 0\n",
     "contact_cutoff out of range"),
    ("force_field baseline\nnumber_of_particles 1000\nlad_fraction 1.5\n",
     "lad_fraction out of range"),
    ("force_field baseline\nnumber_of_particles 1000\nmean_block_length 0.5\n",
     "mean_block_length out of range"),
    # kernels 0 and 1 need cells of the full cutoff (no 5x5x5 stencil)
    ("force_field baseline\nnumber_of_particles 1000\npair_kernel 0\ncell_side 1.25\n",
     "cell_side below interaction cutoff"),
])
def test_parameter_errors_use_ccp_messages(engine_lib, text, msg):
    from tfm_gb300 import ccpgpu

    h = C.c_void_p()
    rc = engine_lib.ccpgpu_create(text.encode(), 0, C.byref(h))
    assert rc == ccpgpu.ERR_PARAM
    assert engine_lib.ccpgpu_last_error().decode() == msg
    assert not h


def test_first_key_occurrence_wins(engine_lib):
    """parmap keeps the first value of a repeated key (std::map::insert)."""
    h = C.c_void_p()
    rc = engine_lib.ccpgpu_create(b"number_of_particles 0\nnumber_of_particles 1000\n"
                                  b"nucleus_radius 10\n", 0, C.byref(h))
    assert engine_lib.ccpgpu_last_error().decode() == "number_of_particles out of range"


def test_null_arguments_are_rejected(engine_lib):
    from tfm_gb300 import ccpgpu

    assert engine_lib.ccpgpu_create(None, 0, None) == ccpgpu.ERR_ARG
    assert engine_lib.ccpgpu_info_get(None, None) == ccpgpu.ERR_ARG


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_pair_lanes_values_parse(engine_lib, lanes):
    """Every documented lanes-per-bead value passes the parameter checks (on a
    machine without a GPU the call then fails at the device, not at them)."""
    from tfm_gb300 import ccpgpu

    h = C.c_void_p()
    text = "force_field baseline\nnumber_of_particles 1000\npair_lanes %d\n" % lanes
    rc = engine_lib.ccpgpu_create(text.encode(), 0, C.byref(h))
    if rc == ccpgpu.OK:
        engine_lib.ccpgpu_destroy(h)
    else:
        assert rc != ccpgpu.ERR_PARAM, engine_lib.ccpgpu_last_error().decode()

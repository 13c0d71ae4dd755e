"""Golden vectors for the per-frame observables of ccp-analyze (the
reference's chrana::calc_observables, Program/src/chrana.cu:371-480): centre
of mass distance, gyration radius squared, nematic order parameter, nucleus
chromatin fraction and the 3 x 64 radial chromatin densities.

Seeded frames are written in ccp's own formats (a .gro initial condition with
the bead types, then a .trr file of frames_per_file FP32 frames) and analysed
by oracle/_ref/chrana_driver, which runs the reference's own analysis code on
the host (built from the reference sources by oracle/ref/build_chrana.sh).
The frames as ccp reads them (the .gro at its 3 printed decimals, the .trr
frames exactly) and the printed series are stored in
tests/golden/observables_ccp.npz.

Cases: a 2048-bead chain in a sphere, and a 4096-bead chain in a nucleus
with an opening and a bleb holding a tenth of the beads (fraction below
1, equal-volume shells cut by the bleb).
Usage: python tests/golden/make_chrana_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "chrana_driver")
RCO = 1.154701


def walk(rng, n, radius, centre=(0.0, 0.0, 0.0)):
    """A unit-step chain kept inside a sphere (rejection of outside steps)."""
    c = np.asarray(centre, np.float64)
    x = np.zeros((n, 3))
    x[0] = c + rng.uniform(-0.5, 0.5, 3)  # off the centre: the order parameter divides by |r|
    for i in range(1, n):
        while True:
            v = rng.normal(size=3)
            p = x[i - 1] + v / np.linalg.norm(v)
            if np.linalg.norm(p - c) < radius:
                x[i] = p
                break
    return x


def gro_text(x, types):
    """ccp's write_frame_txt layout (chrdat.cu:107-133)."""
    n = len(x)
    lines = ["0 0", "%5d" % n]
    for i in range(n):
        c = "A" if types[i] == 0 else "B"
        lines.append("%5d%-5s%5s%5d%8.3f%8.3f%8.3f" % (i + 1, c, c, i + 1, *x[i]))
    lines.append("%10.5f%10.5f%10.5f" % (0.0, 0.0, 0.0))
    return "\n".join(lines) + "\n"


def trr_frame(i_f, t, x):
    """ccp's write_frame_bin layout (chrdat.cu:168-194)."""
    n = len(x)
    hdr = np.zeros(18, np.uint32)
    hdr[0], hdr[1], hdr[10], hdr[13], hdr[14] = 1993, 1, 3 * n * 4, n, i_f
    hdr[16] = np.array([t], np.float32).view(np.uint32)[0]
    return hdr.tobytes() + np.asarray(x, np.float32).tobytes()


def run_case(rng, n, R_n, R_o, R_b, n_frames, bleb_frac):
    types = np.where(rng.random(n) < 0.5, 0, 1).astype(np.int32)
    nod = float(np.sqrt(np.float32(R_n) ** 2 - np.float32(R_o) ** 2))
    bod = float(np.sqrt(np.float32(R_b) ** 2 - np.float32(R_o) ** 2))
    n_bleb = int(bleb_frac * n)
    frames = []
    for k in range(1 + n_frames):
        x = walk(rng, n - n_bleb, R_n - 1.0)
        if n_bleb:
            xb = walk(rng, n_bleb, R_b - 1.0, (0.0, 0.0, nod + bod))
            x = np.concatenate([x, xb])
        frames.append(x.astype(np.float32))
    with tempfile.TemporaryDirectory() as d:
        par = os.path.join(d, "par.dat")
        with open(par, "w") as f:
            f.write("number_of_particles %d\nnucleus_radius %.6f\nopening_radius %.6f\n"
                    "bleb_radius %.6f\nframes_per_file %d\n" % (n, R_n, R_o, R_b, n_frames))
        gro = os.path.join(d, "ic.gro")
        text = gro_text(frames[0], types)
        with open(gro, "w") as f:
            f.write(text)
        trr = os.path.join(d, "traj.trr")
        with open(trr, "wb") as f:
            for k in range(1, 1 + n_frames):
                f.write(trr_frame(k, 0.25 * k, frames[k]))
        out = os.path.join(d, "out.txt")
        subprocess.run([DRIVER, par, gro, trr, out], check=True, capture_output=True)
        vals = np.loadtxt(out, dtype=np.float64, ndmin=2)
    # the initial frame as ccp parsed it: its printed decimals, rounded to FP32
    x0 = np.array([[np.float32(v) for v in ln[20:44].split()] for ln in text.splitlines()[2:2 + n]],
                  np.float32)
    xs = np.stack([x0] + frames[1:])
    return dict(xyz=xs, types=types, R_n=np.float32(R_n), R_o=np.float32(R_o),
                R_b=np.float32(R_b), nod=np.float32(nod), series=vals)


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the driver first: oracle/ref/build_chrana.sh")
    rng = np.random.default_rng(20261204)
    cases = [run_case(rng, 2048, 0.5 * RCO * (1 + (2048 / 0.2) ** (1 / 3)), 0.0, 0.0, 3, 0.0),
             run_case(rng, 4096, 14.0, 4.0, 6.0, 2, 0.1)]
    out = {}
    for k, c in enumerate(cases):
        for key, v in c.items():
            out["c%d_%s" % (k, key)] = v
    np.savez_compressed(os.path.join(HERE, "observables_ccp.npz"), n_cases=len(cases), **out)
    print("wrote %d cases" % len(cases))


if __name__ == "__main__":
    main()

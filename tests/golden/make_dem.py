"""Detector-error-model fixtures written by the REFERENCE's own CLI.

Run where the reference tree exists (it is never copied into this repository):

    make -C oracle ref
    python tests/golden/make_dem.py

For each case it writes tests/golden/dem/<case>.npz with the model text (a hand-written model, or the
reference's `stim analyze_errors` of a generated circuit), the model's detector / observable / error counts
as the reference's `stim sample_dem` reports them (row lengths of its 01 output), recorded errors (seeded
random bits) with the detection events and observable flips the reference's `stim sample_dem
--replay_err_in` gives for them, and the per-detector / per-observable counts of 2^18 shots of the
reference's own sampler (its native RNG) for the statistical agreement tests.  It also writes
tests/golden/dem/surface_rz_d25_r25_p0.001.dem.xz, the reference's `stim analyze_errors` of the d=25,
25-round rotated memory-Z circuit at p = 1e-3 (the benchmark's model).
"""

import lzma
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from stim_gb300 import workloads  # noqa: E402

STIM = os.path.join(ROOT, "oracle", "_ref", "stim")
OUT = os.path.join(HERE, "dem")
RATE_SHOTS = 1 << 18


def run(args):
    return subprocess.run([STIM] + args, check=True, capture_output=True).stdout


def analyze(text):
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "c.stim")
        with open(p, "w") as f:
            f.write(text)
        return run(["analyze_errors", "--in", p]).decode()


def cases():
    cc = workloads.code_circuit
    with open(os.path.join(HERE, "hand", "model.dem")) as f:
        hand = f.read()
    return [
        ("hand", hand, 512),
        ("surface_rz_d3_r3", analyze(cc("surface_code:rotated_memory_z", 3, 3, 0.001)), 256),
        ("surface_rx_d5_r5", analyze(cc("surface_code:rotated_memory_x", 5, 5, 0.01)), 256),
        ("rep_d9_r9", analyze(cc("repetition_code:memory", 9, 9, 0.02)), 256),
        ("color_d5_r5", analyze(cc("color_code:memory_xyz", 5, 5, 0.01)), 200),
    ]


def read_b8(path, shots, n):
    nb = (n + 7) // 8
    return np.frombuffer(open(path, "rb").read(), dtype=np.uint8).reshape(shots, nb)


def main():
    os.makedirs(OUT, exist_ok=True)
    big = analyze(workloads.code_circuit("surface_code:rotated_memory_z", 25, 25, 0.001))
    with lzma.open(os.path.join(OUT, "surface_rz_d25_r25_p0.001.dem.xz"), "wt", preset=9) as f:
        f.write(big)
    rng = np.random.default_rng(77)
    for name, text, shots in cases():
        with tempfile.TemporaryDirectory() as td:
            mpath = os.path.join(td, "m.dem")
            with open(mpath, "w") as f:
                f.write(text)
            p = lambda n: os.path.join(td, n)  # noqa: E731
            run(["sample_dem", "--shots", "1", "--seed", "1", "--in", mpath, "--out", p("d.01"), "--obs_out",
                 p("o.01"), "--err_out", p("e.01")])
            D = len(open(p("d.01")).read().rstrip("\n"))
            O = len(open(p("o.01")).read().rstrip("\n"))
            E = len(open(p("e.01")).read().rstrip("\n"))
            errs = (rng.random((shots, E)) < 0.1)
            packed = np.packbits(errs, axis=1, bitorder="little")
            packed.tofile(p("r.b8"))
            run(["sample_dem", "--shots", str(shots), "--in", mpath, "--replay_err_in", p("r.b8"),
                 "--replay_err_in_format", "b8", "--out", p("d.b8"), "--out_format", "b8", "--obs_out", p("o.b8"),
                 "--obs_out_format", "b8"])
            dets = read_b8(p("d.b8"), shots, D)
            obs = read_b8(p("o.b8"), shots, O)
            run(["sample_dem", "--shots", str(RATE_SHOTS), "--seed", "3", "--in", mpath, "--out", p("rd.b8"),
                 "--out_format", "b8", "--obs_out", p("ro.b8"), "--obs_out_format", "b8"])
            rd = read_b8(p("rd.b8"), RATE_SHOTS, D)
            ro = read_b8(p("ro.b8"), RATE_SHOTS, O)
            det_counts = np.unpackbits(rd, axis=1, bitorder="little")[:, :D].sum(axis=0, dtype=np.int64)
            obs_counts = np.unpackbits(ro, axis=1, bitorder="little")[:, :O].sum(axis=0, dtype=np.int64)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), model=text, num_detectors=D, num_observables=O,
                            num_errors=E, replay=packed, dets=dets, obs=obs, rate_shots=RATE_SHOTS,
                            det_counts=det_counts, obs_counts=obs_counts)
        print(name, D, O, E)


if __name__ == "__main__":
    main()

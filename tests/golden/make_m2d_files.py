"""File fixtures for the converter's convert_file, written by the REFERENCE's own CLI.

Run where the reference tree exists (it is never copied into this repository):

    make -C oracle ref
    python tests/golden/make_m2d_files.py

For each case (a circuit from the m2d / m2d_sweep fixtures) it writes tests/golden/m2d_files/<case>.npz holding,
as byte arrays: 128 shots of measurement records in every result format (ptb64 written by `stim sample`, the
others by `stim convert` from it; the reference cannot write ptb64 through `convert` or `m2d`), sweep records the
same way (sampled from a circuit of fair coin flips), and the reference's `stim m2d` output files for every output
format it can write: detection events with observables appended (`out_<F>`), and detection events plus a separate
observable file (`det_<F>`, `obs_<F>`), reading the b8 inputs.
"""

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from make_golden import STIM  # noqa: E402

OUT = os.path.join(HERE, "m2d_files")
FORMATS = ["01", "b8", "r8", "ptb64", "hits", "dets"]
SHOTS = 128


def run(args):
    subprocess.run([STIM] + args, check=True, capture_output=True)


def main():
    os.makedirs(OUT, exist_ok=True)
    cases = [("surface_rx_d5_r5", os.path.join(HERE, "m2d", "surface_rx_d5_r5.npz")),
             ("basic_swept", os.path.join(HERE, "m2d_sweep", "basic.npz")),
             ("rep_d7_r7_swept", os.path.join(HERE, "m2d_sweep", "rep_d7_r7_swept.npz"))]
    for name, src in cases:
        g = np.load(src)
        text = str(g["circuit"])
        M = int(g["num_measurements"])
        S = int(g["num_sweep_bits"]) if "sweep" in g.files else 0
        files = {}
        with tempfile.TemporaryDirectory() as td:
            p = lambda n: os.path.join(td, n)  # noqa: E731
            with open(p("c.stim"), "w") as f:
                f.write(text)
            with open(p("coins.stim"), "w") as f:
                qs = " ".join(str(q) for q in range(S))
                f.write(f"X_ERROR(0.5) {qs}\nM {qs}\n")

            def records(kind, circuit, nbits):
                run(["sample", "--shots", str(SHOTS), "--seed", "11", "--out_format", "ptb64", "--in", circuit,
                     "--out", p(kind + ".ptb64")])
                run(["convert", "--in", p(kind + ".ptb64"), "--in_format", "ptb64", "--out", p(kind + ".b8"),
                     "--out_format", "b8", "--num_measurements", str(nbits), "--num_detectors", "0",
                     "--num_observables", "0"])
                for fmt in FORMATS:
                    if fmt not in ("ptb64", "b8"):
                        run(["convert", "--in", p(kind + ".b8"), "--in_format", "b8", "--out", p(kind + "." + fmt),
                             "--out_format", fmt, "--num_measurements", str(nbits), "--num_detectors", "0",
                             "--num_observables", "0"])
                    files[kind + "_" + fmt] = open(p(kind + "." + fmt), "rb").read()

            records("meas", p("c.stim"), M)
            sweep_args = []
            if S:
                records("sweep", p("coins.stim"), S)
                sweep_args = ["--sweep", p("sweep.b8"), "--sweep_format", "b8"]
            for fmt in FORMATS:
                if fmt == "ptb64":
                    continue
                base = ["m2d", "--circuit", p("c.stim"), "--in", p("meas.b8"), "--in_format", "b8"] + sweep_args
                run(base + ["--out", p("o"), "--out_format", fmt, "--append_observables"])
                files["out_" + fmt] = open(p("o"), "rb").read()
                run(base + ["--out", p("d"), "--out_format", fmt, "--obs_out", p("l"), "--obs_out_format", fmt])
                files["det_" + fmt] = open(p("d"), "rb").read()
                files["obs_" + fmt] = open(p("l"), "rb").read()
        np.savez_compressed(os.path.join(OUT, name + ".npz"), circuit=text, has_sweep=S > 0,
                            **{k: np.frombuffer(v, dtype=np.uint8) for k, v in files.items()})
        print(name, {k: len(v) for k, v in files.items() if k.startswith("out_")})


if __name__ == "__main__":
    main()

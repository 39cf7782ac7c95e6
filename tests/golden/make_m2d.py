"""Measurements-to-detection-events fixtures written by the REFERENCE's own CLI (`stim m2d`).

Run where the reference tree exists (it is never copied into this repository):

    make -C oracle ref
    python tests/golden/make_m2d.py

For each case it writes tests/golden/m2d/<case>.npz with the circuit text, bit-packed measurement rows
(half sampled by the reference's `stim sample`, half uniformly random bits, so every detector parity
pattern occurs), the reference's `stim m2d --append_observables` output for them (with and without
--skip_reference_sample), and the reference sample from the reference's TableauSimulator
(oracle/_ref/ref_inject).
"""

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from make_golden import REF_INJECT, STIM, hand, run_ref  # noqa: E402
from stim_gb300 import workloads  # noqa: E402

OUT = os.path.join(HERE, "m2d")


def cases():
    cc = workloads.code_circuit
    return [
        ("surface_rz_d3_r3", cc("surface_code:rotated_memory_z", 3, 3, 0.001), 256),
        ("surface_rx_d5_r5", cc("surface_code:rotated_memory_x", 5, 5, 0.01), 300),
        ("rep_d9_r9", cc("repetition_code:memory", 9, 9, 0.02), 256),
        ("color_d5_r5", cc("color_code:memory_xyz", 5, 5, 0.01), 200),
        ("all_gates", hand("all_gates"), 256),
        ("feedback", hand("feedback"), 256),
        ("obs_data", hand("obs_data"), 130),
        ("random_clifford_n64_d60", workloads.random_clifford_circuit(64, 60, 21), 128),
    ]


def run(args):
    subprocess.run([STIM] + args, check=True, capture_output=True)


def main():
    os.makedirs(OUT, exist_ok=True)
    rng = np.random.default_rng(2025)
    for name, text, shots in cases():
        ref = run_ref(text, 1, 64)
        M = ref["num_measurements"]
        mrow = (M + 7) // 8
        with tempfile.TemporaryDirectory() as td:
            cpath = os.path.join(td, "c.stim")
            with open(cpath, "w") as f:
                f.write(text)
            spath = os.path.join(td, "s.b8")
            run(["sample", "--shots", str(shots // 2), "--seed", "7", "--out_format", "b8", "--in", cpath,
                 "--out", spath])
            sampled = np.frombuffer(open(spath, "rb").read(), dtype=np.uint8).reshape(shots // 2, mrow)
            rand = rng.integers(0, 256, size=(shots - shots // 2, mrow), dtype=np.uint8)
            if M % 8:
                rand[:, -1] &= (1 << (M % 8)) - 1
            meas = np.concatenate([sampled, rand])
            mpath = os.path.join(td, "m.b8")
            meas.tofile(mpath)
            outs = {}
            for key, extra in (("out", []), ("out_skip", ["--skip_reference_sample"])):
                opath = os.path.join(td, key + ".b8")
                run(["m2d", "--circuit", cpath, "--in", mpath, "--in_format", "b8", "--out", opath,
                     "--out_format", "b8", "--append_observables"] + extra)
                nb = (ref["num_detectors"] + ref["num_observables"] + 7) // 8
                outs[key] = np.frombuffer(open(opath, "rb").read(), dtype=np.uint8).reshape(shots, nb)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), circuit=text, meas=meas, ref_sample=ref["ref_sample"],
                            num_detectors=ref["num_detectors"], num_observables=ref["num_observables"],
                            num_measurements=M, **outs)
        print(name, meas.shape, outs["out"].shape)


if __name__ == "__main__":
    main()

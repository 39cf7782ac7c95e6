"""Sweep-data fixtures for the measurements-to-detection-events converter, written by the REFERENCE's own CLI
(`stim m2d --sweep ... --sweep_format b8`).

Run where the reference tree exists (it is never copied into this repository):

    make -C oracle ref
    python tests/golden/make_m2d_sweep.py

For each case it writes tests/golden/m2d_sweep/<case>.npz with the circuit text, bit-packed measurement rows
(uniformly random: the converter reads any measurement data), bit-packed sweep rows (uniformly random, the first
rows all zero), the reference sample (oracle/_ref/ref_inject) and the reference's `stim m2d --append_observables`
output for them.
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

from make_golden import STIM, run_ref  # noqa: E402
from stim_gb300 import workloads  # noqa: E402

OUT = os.path.join(HERE, "m2d_sweep")

BASIC = """
CX sweep[0] 0
CY sweep[1] 1
CZ sweep[2] 2
H 2
XCZ 3 sweep[3]
YCZ 4 sweep[1]
CZ 5 sweep[4] sweep[0] 6
H 5 6
CZ sweep[5] sweep[6]
M 0 1 2 3 4 5 6
DETECTOR rec[-7]
DETECTOR rec[-6]
DETECTOR rec[-5]
DETECTOR rec[-4]
DETECTOR rec[-3]
DETECTOR rec[-2] rec[-1]
OBSERVABLE_INCLUDE(0) rec[-1] rec[-7]
R 7
CZ sweep[2] 7
OBSERVABLE_INCLUDE(1) X7
MR 0 1
CX rec[-1] 2 sweep[3] 2
M 2
DETECTOR rec[-1]
"""


def with_sweeps(text, rng, nsweep, every):
    """Inserts sweep-controlled Paulis on random qubits after every `every`-th line outside REPEAT headers."""
    out = []
    qubits = sorted({int(t) for line in text.splitlines() for t in line.split()[1:] if t.isdigit()})
    for k, line in enumerate(text.splitlines()):
        out.append(line)
        s = line.strip()
        if s and not s.endswith("{") and not s.startswith(("DETECTOR", "OBSERVABLE", "SHIFT", "QUBIT", "#"))\
                and k % every == 0:
            g = ["CX", "CY", "CZ"][int(rng.integers(3))]
            q = int(rng.choice(qubits))
            out.append(f"{g} sweep[{int(rng.integers(nsweep))}] {q}")
    return "\n".join(out) + "\n"


def cases(rng):
    cc = workloads.code_circuit
    return [
        ("basic", BASIC, 300),
        ("surface_rz_d3_r3_swept", with_sweeps(cc("surface_code:rotated_memory_z", 3, 3, 0.001), rng, 9, 3), 260),
        ("surface_rx_d5_r5_swept", with_sweeps(cc("surface_code:rotated_memory_x", 5, 5, 0.01), rng, 25, 2), 200),
        ("rep_d7_r7_swept", with_sweeps(cc("repetition_code:memory", 7, 7, 0.02), rng, 7, 2), 256),
        ("random_clifford_n32_d30_swept", with_sweeps(workloads.random_clifford_circuit(32, 30, 5), rng, 16, 2),
         130),
    ]


def run(args):
    subprocess.run([STIM] + args, check=True, capture_output=True)


def main():
    os.makedirs(OUT, exist_ok=True)
    rng = np.random.default_rng(4242)
    for name, text, shots in cases(rng):
        ref = run_ref(text, 1, 64)
        M = ref["num_measurements"]
        S = 1 + max(int(t[len("sweep["):-1]) for t in text.replace("\n", " ").split() if t.startswith("sweep["))
        mrow, srow = (M + 7) // 8, (S + 7) // 8
        meas = rng.integers(0, 256, size=(shots, mrow), dtype=np.uint8)
        if M % 8:
            meas[:, -1] &= (1 << (M % 8)) - 1
        sweep = rng.integers(0, 256, size=(shots, srow), dtype=np.uint8)
        if S % 8:
            sweep[:, -1] &= (1 << (S % 8)) - 1
        sweep[:7] = 0
        with tempfile.TemporaryDirectory() as td:
            cpath = os.path.join(td, "c.stim")
            with open(cpath, "w") as f:
                f.write(text)
            mpath, spath, opath = (os.path.join(td, n) for n in ("m.b8", "s.b8", "o.b8"))
            meas.tofile(mpath)
            sweep.tofile(spath)
            run(["m2d", "--circuit", cpath, "--in", mpath, "--in_format", "b8", "--sweep", spath, "--sweep_format",
                 "b8", "--out", opath, "--out_format", "b8", "--append_observables"])
            nb = (ref["num_detectors"] + ref["num_observables"] + 7) // 8
            out = np.frombuffer(open(opath, "rb").read(), dtype=np.uint8).reshape(shots, nb)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), circuit=text, meas=meas, sweep=sweep,
                            num_sweep_bits=S, ref_sample=ref["ref_sample"], num_detectors=ref["num_detectors"],
                            num_observables=ref["num_observables"], num_measurements=M, out=out)
        print(name, meas.shape, sweep.shape, out.shape)


if __name__ == "__main__":
    main()

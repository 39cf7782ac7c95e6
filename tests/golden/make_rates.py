"""Per-detector and per-observable flip counts of the REFERENCE's own CPU sampler (its native
std::mt19937_64 stream, `stim detect`), for the statistical agreement tests of the native-RNG GPU path.

Run where the reference tree exists (it is never copied into this repository):

    make -C oracle ref                 # builds oracle/_ref/stim from the reference's own sources
    python tests/golden/make_rates.py

It writes tests/golden/rates/<case>.npz with the circuit text, shot count, seed and the number of shots in
which each detector (and each observable) fired.
"""

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
OUT = os.path.join(HERE, "rates")
SHOTS = 1 << 18


def cases():
    cc = workloads.code_circuit
    with open(os.path.join(HERE, "hand", "all_gates.stim")) as f:
        all_gates = f.read()
    with open(os.path.join(HERE, "hand", "pauli_channels.stim")) as f:
        channels = f.read()
    return [
        ("surface_rz_d5_r5_p0.01", cc("surface_code:rotated_memory_z", 5, 5, 0.01), 11),
        ("surface_rx_d11_r11_p0.005", cc("surface_code:rotated_memory_x", 11, 11, 0.005), 12),
        ("rep_d9_r9_p0.02", cc("repetition_code:memory", 9, 9, 0.02), 13),
        ("color_d5_r5_p0.01", cc("color_code:memory_xyz", 5, 5, 0.01), 14),
        ("all_gates", all_gates, 15),
        ("pauli_channels", channels, 16),
    ]


def counts(text, seed, shots):
    with tempfile.TemporaryDirectory() as td:
        cpath = os.path.join(td, "c.stim")
        dpath = os.path.join(td, "d.b8")
        opath = os.path.join(td, "o.b8")
        with open(cpath, "w") as f:
            f.write(text)
        subprocess.run([STIM, "detect", "--in", cpath, "--shots", str(shots), "--seed", str(seed), "--out", dpath,
                        "--out_format", "b8", "--obs_out", opath, "--obs_out_format", "b8"], check=True)
        from stim_gb300 import Circuit

        c = Circuit(text)
        D, O = c.num_detectors, c.num_observables
        d = np.fromfile(dpath, dtype=np.uint8).reshape(shots, (D + 7) // 8) if D else np.zeros((shots, 0), np.uint8)
        o = np.fromfile(opath, dtype=np.uint8).reshape(shots, (O + 7) // 8) if O else np.zeros((shots, 0), np.uint8)
        dc = np.unpackbits(d, axis=1, bitorder="little")[:, :D].sum(axis=0, dtype=np.int64)
        oc = np.unpackbits(o, axis=1, bitorder="little")[:, :O].sum(axis=0, dtype=np.int64)
        return dc, oc


def main():
    os.makedirs(OUT, exist_ok=True)
    for name, text, seed in cases():
        dc, oc = counts(text, seed, SHOTS)
        np.savez_compressed(os.path.join(OUT, name + ".npz"), circuit=np.array(text), shots=np.int64(SHOTS),
                            seed=np.int64(seed), det_counts=dc, obs_counts=oc)
        print(name, len(dc), len(oc), dc.sum(), oc.sum())


if __name__ == "__main__":
    main()

"""Regenerates the golden fixtures under tests/golden/ from the REFERENCE itself.

Run in a container where the reference tree exists (it is never copied into this repository):

    make -C oracle ref                 # builds oracle/_ref/stim and oracle/_ref/ref_inject from the
                                       # reference's own sources
    python tests/golden/make_golden.py                 # everything
    python tests/golden/make_golden.py --only=NAME     # one sampling fixture (repeatable)

It writes
  * tests/golden/circuits/*.stim  circuits made by the reference's generator (`stim gen`) with all four
                                  noise knobs at 0.001 (stim_gb300.workloads substitutes other p);
  * tests/golden/refsample_random.npz  reference samples (the reference's TableauSimulator) of 300 random
                                  small circuits mixing every sign-sensitive gate family;
  * tests/golden/refsample_multi.npz   the same for 300 random circuits whose measurements, resets and pair
                                  measurements take several targets at once (the reference collapses an
                                  instruction's X / Y targets in ascending qubit order, which decides the
                                  random outcomes forced to 0);
  * tests/golden/<case>.npz       for each case: the circuit text, seed, shot count, and the
                                  detection events, observable flips and measurement flips that the
                                  reference's FrameSimulator produced when fed the injected random
                                  stream of stim_gb300/csrc/gfs_contract.h (oracle/ref_inject.cc), plus
                                  the reference sample from the reference's TableauSimulator.
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
REF_INJECT = os.path.join(ROOT, "oracle", "_ref", "ref_inject")

GEN = {
    "surface_code:rotated_memory_z": ("surface_code", "rotated_memory_z", list(range(3, 27, 2))),
    "surface_code:rotated_memory_x": ("surface_code", "rotated_memory_x", list(range(3, 23, 2))),
    "surface_code:unrotated_memory_z": ("surface_code", "unrotated_memory_z", [3, 5]),
    "repetition_code:memory": ("repetition_code", "memory", list(range(3, 53, 2))),
    "color_code:memory_xyz": ("color_code", "memory_xyz", list(range(3, 17, 2))),
}


def gen_templates():
    os.makedirs(workloads.CIRCUIT_DIR, exist_ok=True)
    p = workloads.TEMPLATE_P
    for family, (code, task, ds) in GEN.items():
        for d in ds:
            out = subprocess.run(
                [STIM, "gen", "--code", code, "--task", task, "--distance", str(d), "--rounds", str(d),
                 "--after_clifford_depolarization", p, "--before_round_data_depolarization", p,
                 "--before_measure_flip_probability", p, "--after_reset_flip_probability", p],
                check=True, capture_output=True, text=True).stdout
            with open(workloads.template_path(family, d, d), "w") as f:
                f.write(out)


def run_ref(text: str, seed: int, shots: int):
    with tempfile.TemporaryDirectory() as td:
        cpath = os.path.join(td, "c.stim")
        opath = os.path.join(td, "o.bin")
        with open(cpath, "w") as f:
            f.write(text)
        subprocess.run([REF_INJECT, cpath, str(seed), str(shots), opath], check=True)
        raw = open(opath, "rb").read()
    assert raw[:8] == b"GFSREF01"
    s, D, O, M = [int(v) for v in np.frombuffer(raw[8:40], dtype=np.uint64)]
    off = 40
    out = {}
    for name, n in (("dets", D), ("obs", O), ("meas", M)):
        nb = (n + 7) // 8
        out[name] = np.frombuffer(raw[off:off + s * nb], dtype=np.uint8).reshape(s, nb).copy()
        off += s * nb
    out["ref_sample"] = np.frombuffer(raw[off:off + (M + 7) // 8], dtype=np.uint8).copy()
    out["num_detectors"], out["num_observables"], out["num_measurements"] = D, O, M
    return out


def hand(name):
    with open(os.path.join(HERE, "hand", name + ".stim")) as f:
        return f.read()


def cases():
    cc = workloads.code_circuit
    rc = workloads.random_clifford_circuit
    return [
        ("surface_rz_d3_r3_p0.001", cc("surface_code:rotated_memory_z", 3, 3, 0.001), 0, 4096),
        ("surface_rz_d3_r3_p0.05", cc("surface_code:rotated_memory_z", 3, 3, 0.05), 1, 1024),
        ("surface_rx_d5_r5_p0.01", cc("surface_code:rotated_memory_x", 5, 5, 0.01), 2, 1024),
        ("surface_rx_d11_r11_p0.005", cc("surface_code:rotated_memory_x", 11, 11, 0.005), 3, 512),
        ("surface_rx_d11_r11_p0", cc("surface_code:rotated_memory_x", 11, 11, 0.0), 4, 256),
        ("surface_uz_d5_r5_p0.02", cc("surface_code:unrotated_memory_z", 5, 5, 0.02), 5, 512),
        ("rep_d9_r9_p0.02", cc("repetition_code:memory", 9, 9, 0.02), 6, 1024),
        ("color_d5_r5_p0.01", cc("color_code:memory_xyz", 5, 5, 0.01), 7, 1024),
        ("all_gates_s5", hand("all_gates"), 5, 1024),
        ("all_gates_s6_384", hand("all_gates"), 6, 384),
        ("all_gates_s7_200", hand("all_gates"), 7, 200),
        ("feedback", hand("feedback"), 8, 1024),
        ("pauli_channels", hand("pauli_channels"), 9, 1024),
        ("obs_data_1001", hand("obs_data"), 10, 1001),
        ("fusion", hand("fusion"), 15, 1024),
        ("fusion_200", hand("fusion"), 16, 200),
        ("random_clifford_n64_d200_s1", rc(64, 200, 1), 11, 512),
        ("random_clifford_n64_d200_s2", rc(64, 200, 2), 12, 512),
        ("random_clifford_n128_d200_s3", rc(128, 200, 3), 13, 256),
        ("random_clifford_n300_d60_s4", rc(300, 60, 4), 14, 256),
        # The configured random-Clifford sizes (n = 256 and 512 qubits, depth 200).
        ("random_clifford_n256_d200_s25", rc(256, 200, 25), 25, 256),
        ("random_clifford_n512_d200_s26", rc(512, 200, 26), 26, 256),
        # The benchmarked circuit itself: distance 25, 25 rounds, p = 1e-3 (one CTA block per 128 shots,
        # measurement ring in global memory, every randomization removed by the lowering's analysis).
        ("surface_rz_d25_r25_p0.001", cc("surface_code:rotated_memory_z", 25, 25, 0.001), 0, 1024),
    ]


def random_small_circuit(rng, n=4, depth=25):
    """A random small circuit over the gate families whose signs matter for the reference sample: Pauli
    and Clifford gates, measurements and resets in three bases with inverted targets, MPP / SPP / SPP_DAG
    products, pair measurements, classically controlled Paulis, MPAD, heralded erasure, noisy gates."""
    g1 = ["H", "S", "S_DAG", "SQRT_X", "SQRT_Y_DAG", "C_XYZ", "H_YZ", "X", "Y", "Z"]
    g2 = ["CX", "CZ", "CY", "ISWAP", "SQRT_ZZ_DAG", "XCY", "YCZ", "SWAP", "CXSWAP"]
    lines = []
    nmeas = 0

    def term(q):
        return f"{'!' if rng.random() < 0.3 else ''}{rng.choice('XYZ')}{q}"

    for _ in range(depth):
        k = rng.randrange(12)
        qs = list(range(n))
        rng.shuffle(qs)
        if k == 0:
            lines.append(f"{rng.choice(g1)} {qs[0]} {qs[1]}")
        elif k == 1:
            lines.append(f"{rng.choice(g2)} {qs[0]} {qs[1]}")
        elif k == 2:
            lines.append(f"{rng.choice(['M', 'MX', 'MY', 'MR', 'MRX', 'MRY'])} {'!' if rng.random() < 0.3 else ''}{qs[0]}")
            nmeas += 1
        elif k == 3:
            lines.append(f"{rng.choice(['R', 'RX', 'RY'])} {qs[0]}")
        elif k == 4:
            lines.append("MPP " + "*".join(term(q) for q in qs[:rng.randint(1, 3)]))
            nmeas += 1
        elif k == 5:
            lines.append(f"{rng.choice(['SPP', 'SPP_DAG'])} " + "*".join(term(q) for q in qs[:rng.randint(1, 3)]))
        elif k == 6:
            lines.append(f"{rng.choice(['MXX', 'MYY', 'MZZ'])} {'!' if rng.random() < 0.3 else ''}{qs[0]} {qs[1]}")
            nmeas += 1
        elif k == 7 and nmeas:
            g = rng.choice(["CX", "CZ", "CY"])
            lines.append(f"{g} rec[-{rng.randint(1, nmeas)}] {qs[0]}")
        elif k == 8 and nmeas:
            lines.append(f"{rng.choice(['XCZ', 'YCZ'])} {qs[0]} rec[-{rng.randint(1, nmeas)}]")
        elif k == 9:
            lines.append(f"MPAD {rng.randint(0, 1)}")
            nmeas += 1
        elif k == 10:
            lines.append(f"HERALDED_ERASE(0.1) {qs[0]}")
            nmeas += 1
        elif k == 11:
            lines.append(f"X_ERROR(0.2) {qs[0]}\nM(0.1) {qs[1]}")
            nmeas += 1
    return "\n".join(lines) + "\n"


def random_multi_target_circuit(rng, n=6, depth=14):
    """A random circuit whose measurements, resets and pair measurements act on several (shuffled) targets of
    entangled qubits at once, with MPP products in several disjoint and overlapping groups."""
    g1 = ["H", "S", "SQRT_X", "C_XYZ", "H_YZ", "X", "Y"]
    g2 = ["CX", "CZ", "CY", "ISWAP", "SQRT_XX", "XCY", "SWAP"]
    lines = []
    nmeas = 0
    for _ in range(depth):
        k = rng.randrange(8)
        qs = list(range(n))
        rng.shuffle(qs)
        m = rng.randint(2, n)
        if k == 0:
            lines.append(f"{rng.choice(g1)} " + " ".join(map(str, qs[:m])))
        elif k == 1:
            lines.append(f"{rng.choice(g2)} " + " ".join(map(str, qs[:2 * (m // 2)])))
        elif k == 2:
            g = rng.choice(["M", "MX", "MY", "MR", "MRX", "MRY"])
            lines.append(f"{g} " + " ".join(("!" if rng.random() < 0.3 else "") + str(q) for q in qs[:m]))
            nmeas += m
        elif k == 3:
            lines.append(f"{rng.choice(['R', 'RX', 'RY'])} " + " ".join(map(str, qs[:m])))
        elif k == 4:
            pairs = qs[:2 * (m // 2)]
            extra = rng.sample(range(n), 2)  # a repeated qubit starts a new disjoint run
            tgts = pairs + extra
            lines.append(f"{rng.choice(['MXX', 'MYY', 'MZZ'])} " + " ".join(map(str, tgts)))
            nmeas += len(tgts) // 2
        elif k == 5:
            prods = []
            for _ in range(rng.randint(2, 4)):
                sub = rng.sample(range(n), rng.randint(1, 3))
                prods.append("*".join(f"{rng.choice('XYZ')}{q}" for q in sub))
            lines.append("MPP " + " ".join(prods))
            nmeas += len(prods)
        elif k == 6 and nmeas:
            lines.append(f"{rng.choice(['CX', 'CZ', 'CY'])} rec[-{rng.randint(1, nmeas)}] {qs[0]}")
        else:
            lines.append(f"{rng.choice(['SPP', 'SPP_DAG'])} " + "*".join(f"{rng.choice('XYZ')}{q}" for q in qs[:3]))
    return "\n".join(lines) + "\n"


def refsample_fixtures(count=300, seed=3, make=random_small_circuit, name="refsample_random.npz"):
    """Reference samples (the reference's TableauSimulator) of random small circuits."""
    import random

    rng = random.Random(seed)
    texts, samples = [], []
    while len(texts) < count:
        text = make(rng)
        try:
            out = run_ref(text, 1, 128)
        except subprocess.CalledProcessError:
            continue  # a combination the reference rejects
        texts.append(text)
        samples.append(out["ref_sample"])
    width = max(len(s) for s in samples)
    packed = np.zeros((len(samples), width), dtype=np.uint8)
    lengths = np.array([len(s) for s in samples], dtype=np.int64)
    for k, s in enumerate(samples):
        packed[k, :len(s)] = s
    np.savez_compressed(os.path.join(HERE, name), circuits=np.array(texts), samples=packed,
                        lengths=lengths, seed=np.uint64(seed))


def main():
    if "--refsample-only" in sys.argv:
        refsample_fixtures()
        return
    if "--refsample-multi-only" in sys.argv:
        refsample_fixtures(seed=5, make=random_multi_target_circuit, name="refsample_multi.npz")
        return
    only = [a.split("=", 1)[1] for a in sys.argv[1:] if a.startswith("--only=")]
    if not only:
        gen_templates()
    for name, text, seed, shots in cases():
        if only and name not in only:
            continue
        out = run_ref(text, seed, shots)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), circuit=np.array(text), seed=np.uint64(seed),
                            shots=np.uint64(shots), **out)
        print(name, out["num_detectors"], out["num_measurements"], shots)
    if not only:
        refsample_fixtures()
        refsample_fixtures(seed=5, make=random_multi_target_circuit, name="refsample_multi.npz")


if __name__ == "__main__":
    main()

"""Synthetic circuit workloads.

* ``code_circuit(family, distance, rounds, p)`` loads a committed circuit of one of the reference's
  generated code families (rotated/unrotated surface code, repetition code, color code), produced by
  the reference's own generator with all four noise knobs (after_clifford_depolarization,
  before_round_data_depolarization, before_measure_flip_probability, after_reset_flip_probability)
  set to 0.001, and substitutes the requested probability.  The templates live in
  tests/golden/circuits/ and are made by tests/golden/make_golden.py.
* ``random_clifford_circuit`` builds the random-Clifford correctness workload: layers drawn uniformly
  from {H, S, CX, CZ, SWAP, ISWAP, MPP (2-4 body), M, R, MR}, DEPOLARIZE1/2 after each gate layer with
  p in [1e-4, 1e-2], and every measurement result annotated as its own DETECTOR.
"""

import math
import os
import random

_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CIRCUIT_DIR = os.path.join(_ROOT, "tests", "golden", "circuits")

FAMILIES = {
    "surface_code:rotated_memory_z": "surface_rz",
    "surface_code:rotated_memory_x": "surface_rx",
    "surface_code:unrotated_memory_z": "surface_uz",
    "repetition_code:memory": "rep",
    "color_code:memory_xyz": "color",
}

TEMPLATE_P = "0.001"


def template_path(family: str, distance: int, rounds: int) -> str:
    return os.path.join(CIRCUIT_DIR, f"{FAMILIES[family]}_d{distance}_r{rounds}.stim")


def format_p(p: float) -> str:
    if p == 0:
        return "0"
    s = repr(float(p))
    return s


def code_circuit(family: str, distance: int, rounds: int, p: float) -> str:
    """The generated code circuit with every noise probability set to p."""
    path = template_path(family, distance, rounds)
    if not os.path.exists(path):
        raise FileNotFoundError(f"no committed template for {family} d={distance} r={rounds}: {path}")
    with open(path) as f:
        text = f.read()
    return text.replace("(" + TEMPLATE_P + ")", "(" + format_p(p) + ")")


def dem_d25_text() -> str:
    """The reference's `stim analyze_errors` of the d=25, 25-round rotated memory-Z circuit at p = 1e-3
    (15,600 detectors, 1 observable, 326,897 error mechanisms), written by tests/golden/make_dem.py."""
    import lzma

    with lzma.open(os.path.join(_ROOT, "tests", "golden", "dem", "surface_rz_d25_r25_p0.001.dem.xz"), "rt") as f:
        return f.read()


def random_clifford_circuit(num_qubits: int, depth: int, seed: int, p_lo: float = 1e-4,
                            p_hi: float = 1e-2) -> str:
    rng = random.Random(seed)
    gates = ["H", "S", "CX", "CZ", "SWAP", "ISWAP", "MPP", "M", "R", "MR"]
    lines = []

    def p_draw():
        return math.exp(rng.uniform(math.log(p_lo), math.log(p_hi)))

    def subset():
        return [q for q in range(num_qubits) if rng.random() < 0.5]

    def pairs():
        qs = list(range(num_qubits))
        rng.shuffle(qs)
        k = rng.randint(1, num_qubits // 2)
        return [(qs[2 * i], qs[2 * i + 1]) for i in range(k)]

    for _ in range(depth):
        g = gates[rng.randrange(len(gates))]
        if g in ("H", "S"):
            qs = subset()
            if not qs:
                continue
            lines.append(g + " " + " ".join(map(str, qs)))
            lines.append(f"DEPOLARIZE1({p_draw():.6g}) " + " ".join(map(str, qs)))
        elif g in ("CX", "CZ", "SWAP", "ISWAP"):
            ps = pairs()
            flat = " ".join(f"{a} {b}" for a, b in ps)
            lines.append(g + " " + flat)
            lines.append(f"DEPOLARIZE2({p_draw():.6g}) " + flat)
        elif g == "MPP":
            qs = list(range(num_qubits))
            rng.shuffle(qs)
            prods = []
            i = 0
            while i + 4 <= len(qs) and rng.random() < 0.9:
                w = rng.randint(2, 4)
                terms = [rng.choice("XYZ") + str(q) for q in qs[i:i + w]]
                i += w
                prods.append(("!" if rng.random() < 0.25 else "") + "*".join(terms))
            if not prods:
                continue
            lines.append("MPP " + " ".join(prods))
            n = len(prods)
            for k in range(n):
                lines.append(f"DETECTOR rec[-{n - k}]")
        else:
            qs = subset()
            if not qs:
                continue
            lines.append(g + " " + " ".join(map(str, qs)))
            if g in ("M", "MR"):
                n = len(qs)
                for k in range(n):
                    lines.append(f"DETECTOR rec[-{n - k}]")
    return "\n".join(lines) + "\n"


def batched_workload(num_circuits: int = 256, seed: int = 2024, d_choices=tuple(range(3, 19, 2)),
                     p_lo: float = 1e-4, p_hi: float = 1e-2, shots_lo: int = 1 << 12, shots_hi: int = 1 << 20):
    """The many-circuit workload: rotated surface-code memory-Z circuits with d drawn uniformly from
    d_choices and rounds = d, p log-uniform in [p_lo, p_hi], shot counts log-uniform in [shots_lo,
    shots_hi], and one sampling seed per circuit; all draws come from a generator seeded with `seed`.
    Returns a list of dicts with keys text, distance, p, shots, seed."""
    rng = random.Random(seed)
    out = []
    for _ in range(num_circuits):
        d = d_choices[rng.randrange(len(d_choices))]
        p = math.exp(rng.uniform(math.log(p_lo), math.log(p_hi)))
        p = float(f"{p:.4g}")
        shots = int(round(math.exp(rng.uniform(math.log(shots_lo), math.log(shots_hi)))))
        out.append({"text": code_circuit("surface_code:rotated_memory_z", d, d, p), "distance": d, "p": p,
                    "shots": shots, "seed": rng.randrange(1 << 62)})
    return out


SERVING_FAMILIES = (
    ("repetition_code:memory", tuple(range(3, 53, 2))),
    ("surface_code:rotated_memory_x", tuple(range(3, 23, 2))),
    ("surface_code:rotated_memory_z", tuple(range(3, 23, 2))),
    ("color_code:memory_xyz", tuple(range(3, 17, 2))),
)


def serving_workload(rate: float = 2000.0, seconds: float = 60.0, seed: int = 7, p_lo: float = 1e-4,
                     p_hi: float = 1e-2, p_per_decade: int = 16, shots_lo: int = 1 << 10, shots_hi: int = 1 << 22):
    """The request-serving workload: Poisson arrivals at `rate` requests per second for `seconds`; each
    request picks a family uniformly, then d uniformly from the family's range (rounds = d), p log-uniform
    in [p_lo, p_hi] rounded to one of `p_per_decade` log-spaced values per decade (so that repeated
    circuits can hit the device-side circuit cache), shots log-uniform in [shots_lo, shots_hi], and its
    own seed.  Returns a list of dicts with keys t (arrival, seconds), family, distance, p, shots, seed."""
    rng = random.Random(seed)
    out = []
    t = 0.0
    lo, hi = math.log10(p_lo), math.log10(p_hi)
    steps = max(1, int(round((hi - lo) * p_per_decade)))
    while True:
        t += rng.expovariate(rate)
        if t >= seconds:
            break
        fam, ds = SERVING_FAMILIES[rng.randrange(len(SERVING_FAMILIES))]
        d = ds[rng.randrange(len(ds))]
        k = rng.randint(0, steps)
        p = float(f"{10 ** (lo + (hi - lo) * k / steps):.4g}")
        shots = int(round(math.exp(rng.uniform(math.log(shots_lo), math.log(shots_hi)))))
        out.append({"t": t, "family": fam, "distance": d, "p": p, "shots": shots, "seed": rng.randrange(1 << 62)})
    return out

"""Signs of every unitary gate's Heisenberg images in the host reference sample, against the reference's own tableau
data (tests/golden/gate_tableaus.txt, written from the reference's GATE_DATA by tests/golden/make_gate_tableaus.py).
Frames carry no signs, but the reference sample (the noiseless run that measurement results are reported against,
the reference's TableauSimulator) does: prepare the +1 eigenstate of a generator (X with RX, Z with R), apply the
gate, and measure the generator's image as a Pauli product; the result is 1 exactly when the image's sign is minus.
Host code (no GPU)."""

import os

import pytest

import stim_gb300

HERE = os.path.dirname(os.path.abspath(__file__))
GATES = [line.split() for line in open(os.path.join(HERE, "golden", "gate_tableaus.txt")) if line.startswith("T ")]


def product(image):
    """'+X_Z' -> 'X0*Z2' (identity factors dropped; an all-identity image has no product)."""
    terms = [f"{p}{q}" for q, p in enumerate(image[1:]) if p != "_"]
    return "*".join(terms)


@pytest.mark.parametrize("row", GATES, ids=[r[1] for r in GATES])
def test_reference_sample_signs_match_reference_tableau(row):
    name, n, images = row[1], int(row[2]), row[3:]
    targets = " ".join(str(q) for q in range(n))
    for k, image in enumerate(images):
        q, basis = k // 2, "X" if k % 2 == 0 else "Z"
        resets = "".join(f"{'RX' if (p == q and basis == 'X') else 'R'} {p}\n" for p in range(n))
        prod = product(image)
        assert prod, f"{name}: empty image"
        c = stim_gb300.Circuit(f"{resets}{name} {targets}\nMPP {prod}")
        got = int(c.reference_sample()[-1])
        assert got == (image[0] == "-"), f"{name}: image of {basis}{q} is {image}, reference sample gave {got}"

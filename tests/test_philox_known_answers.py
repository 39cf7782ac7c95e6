"""The random-bit contract's generator (stim_gb300/csrc/gfs_contract.h gfs_philox, shared by the kernels and the
oracle) against the published known answers of Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as
1, 2, 3", SC11; the Random123 distribution's test vectors for zero, all-ones and pi-digit keys and counters).  The
oracle and the product read the same header, so this pins the generator itself.  CPU, compiled with the host C
compiler."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "stim_gb300", "csrc")

# (key0, key1, counter0..3) -> output words
KNOWN = [
    ((0, 0, 0, 0, 0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 6, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0xA4093822, 0x299F31D0, 0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]

PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include "gfs_contract.h"
int main(int argc, char **argv) {
    unsigned v[6];
    for (int k = 0; k < 6; k++) v[k] = (unsigned)strtoul(argv[1 + k], 0, 16);
    gfs_u32x4 r = gfs_philox(v[0], v[1], v[2], v[3], v[4], v[5]);
    printf("%08x %08x %08x %08x\n", r.v[0], r.v[1], r.v[2], r.v[3]);
    return 0;
}
"""


@pytest.fixture(scope="module")
def philox(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("philox")
    src, exe = d / "kat.c", d / "kat"
    src.write_text(PROGRAM)
    subprocess.run([cc, "-std=c11", "-O1", "-I", CSRC, str(src), "-o", str(exe), "-lm"], check=True)
    return str(exe)


@pytest.mark.parametrize("inputs,want", KNOWN)
def test_philox4x32_10_known_answers(philox, inputs, want):
    out = subprocess.run([philox] + [f"{v:08x}" for v in inputs], capture_output=True, text=True, check=True)
    assert out.stdout.split() == [f"{w:08x}" for w in want]
